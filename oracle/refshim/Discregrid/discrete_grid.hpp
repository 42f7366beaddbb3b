// Discregrid/discrete_grid.hpp — declaration-only stand-in for the Discregrid library (the
// reference fetches it at configure time, commit 0b69062ff9c56fbb6dcecd296652028bedbacf0e,
// CMake/SetUpExternalProjects.cmake:13-20). Test infrastructure only. Its signed-distance
// maps serve the Koschier2017 and Bender2019 boundary methods, which the DiffDFSPH path
// does not use; the reference's sources still name the type, so it is declared here with
// the member functions they call, and nothing defines them: the pin driver never creates
// a map, and linking leaves these symbols unresolved.
#pragma once
#include <Eigen/Dense>
#include <array>

namespace Discregrid {

class DiscreteGrid {
 public:
  virtual ~DiscreteGrid() {}
  double interpolate(unsigned int field_id, Eigen::Vector3d const &xi, Eigen::Vector3d *gradient = nullptr) const;
  double interpolate(unsigned int field_id, Eigen::Vector3d const &xi, const std::array<unsigned int, 32> &cell,
                     const Eigen::Vector3d &c0, const Eigen::Matrix<double, 32, 1> &N,
                     Eigen::Vector3d *gradient = nullptr, Eigen::Matrix<double, 32, 3> *dN = nullptr) const;
  bool determineShapeFunctions(unsigned int field_id, Eigen::Vector3d const &x, std::array<unsigned int, 32> &cell,
                               Eigen::Vector3d &c0, Eigen::Matrix<double, 32, 1> &N,
                               Eigen::Matrix<double, 32, 3> *dN = nullptr) const;
};

}  // namespace Discregrid
