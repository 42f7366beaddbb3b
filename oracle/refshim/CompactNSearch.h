// CompactNSearch.h — a stand-in for the CompactNSearch library (the reference fetches it
// at configure time, commit 3f11ece16a419fc1cc5795d6aa87cb7fe6b86960,
// CMake/NeighborhoodSearch.cmake:32-39). Test infrastructure only: it lets the reference's
// own hot-path sources compile into the reference pin driver (oracle/build_ref_step.sh).
//
// It restates the library's published interface as the reference calls it
// (Simulation.cpp:209-215,743-777,831-900; Simulation.h:398-539; FluidModel.cpp:348;
// BoundaryModel_Akinci2012.cpp:374): point sets over caller-owned coordinate arrays, an
// activation table (set i searches set j), fixed-radius neighbour lists per (i, j), and the
// z-sort hooks. Two choices are this file's own and are the ones the CPU oracle and the GPU
// library make too, so that all three sum neighbours in the same order:
//   - a point b of set j is a neighbour of point a of set i when
//     ((dx*dx + dy*dy) + dz*dz) < r*r, evaluated without contraction (build with
//     -ffp-contract=off), and a point is not its own neighbour;
//   - every list is in ascending index order.
// z_sort() keeps the identity order (the library would reorder the particles in Morton
// order every 500 steps; the pin driver turns z-sorting off as well).
#pragma once
#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <unordered_map>
#include <vector>

namespace CompactNSearch {

#ifdef USE_DOUBLE
typedef double Real;
#else
typedef float Real;
#endif

class NeighborhoodSearch;

class PointSet {
 public:
  PointSet(Real const *x, std::size_t n, bool dynamic, void *user_data)
      : m_x(x), m_n(n), m_dynamic(dynamic), m_user_data(user_data) {}

  std::size_t n_neighbors(unsigned int point_set, unsigned int i) const {
    return point_set < m_neighbors.size() && i < m_neighbors[point_set].size() ? m_neighbors[point_set][i].size() : 0;
  }
  unsigned int neighbor(unsigned int point_set, unsigned int i, unsigned int k) const {
    return m_neighbors[point_set][i][k];
  }
  const std::vector<unsigned int> &neighbor_list(unsigned int point_set, unsigned int i) const {
    return m_neighbors[point_set][i];
  }
  std::size_t n_points() const { return m_n; }
  bool is_dynamic() const { return m_dynamic; }
  void set_dynamic(bool v) { m_dynamic = v; }
  void *get_user_data() { return m_user_data; }
  Real const *point(unsigned int i) const { return &m_x[3 * i]; }
  // the z-sort permutation is the identity, so sorting a field leaves it unchanged
  template <typename T> void sort_field(T *) const {}

 private:
  friend class NeighborhoodSearch;
  Real const *m_x;
  std::size_t m_n;
  bool m_dynamic;
  void *m_user_data;
  std::vector<std::vector<std::vector<unsigned int>>> m_neighbors;  // [other set][point] -> list
};

class NeighborhoodSearch {
 public:
  explicit NeighborhoodSearch(Real r, bool erase_empty_cells = false) : m_r(r) { (void)erase_empty_cells; }

  unsigned int add_point_set(Real const *x, std::size_t n, bool is_dynamic = true, bool search_neighbors = true,
                             bool find_neighbors = true, void *user_data = nullptr) {
    const std::size_t s = m_sets.size();
    for (auto &row : m_active) row.push_back((unsigned char)find_neighbors);
    m_active.emplace_back(s + 1, (unsigned char)search_neighbors);
    m_sets.emplace_back(x, n, is_dynamic, user_data);
    return (unsigned int)s;
  }
  void resize_point_set(unsigned int i, Real const *x, std::size_t n) {
    m_sets[i].m_x = x;
    m_sets[i].m_n = n;
  }
  PointSet const &point_set(unsigned int i) const { return m_sets[i]; }
  PointSet &point_set(unsigned int i) { return m_sets[i]; }
  std::size_t n_point_sets() const { return m_sets.size(); }
  std::vector<PointSet> const &point_sets() const { return m_sets; }
  std::vector<PointSet> &point_sets() { return m_sets; }
  Real radius() const { return m_r; }
  void set_radius(Real r) { m_r = r; }

  bool is_active(unsigned int i, unsigned int j) const { return m_active[i][j] != 0; }
  void set_active(unsigned int i, unsigned int j, bool active) { m_active[i][j] = (unsigned char)active; }
  void set_active(bool active) {
    for (auto &row : m_active) std::fill(row.begin(), row.end(), (unsigned char)active);
  }
  // set `index` searches every set (search_neighbors) and every set searches `index`
  // (find_neighbors)
  void set_active(unsigned int index, bool search_neighbors, bool find_neighbors) {
    for (std::size_t j = 0; j < m_active.size(); j++) {
      m_active[j][index] = (unsigned char)find_neighbors;
      m_active[index][j] = (unsigned char)search_neighbors;
    }
    m_active[index][index] = (unsigned char)(search_neighbors && find_neighbors);
  }
  void update_point_sets() {}
  void update_activation_table() {}
  void z_sort() {}

  void find_neighbors(bool points_changed = true) {
    (void)points_changed;
    const std::size_t ns = m_sets.size();
    for (std::size_t i = 0; i < ns; i++) {
      PointSet &A = m_sets[i];
      A.m_neighbors.assign(ns, std::vector<std::vector<unsigned int>>());
      for (std::size_t j = 0; j < ns; j++) A.m_neighbors[j].assign(A.m_n, std::vector<unsigned int>());
    }
    for (std::size_t j = 0; j < ns; j++) {
      bool wanted = false;
      for (std::size_t i = 0; i < ns; i++) wanted = wanted || m_active[i][j];
      if (!wanted || m_sets[j].m_n == 0) continue;
      Grid g;
      build_grid(m_sets[j], g);
      for (std::size_t i = 0; i < ns; i++) {
        if (!m_active[i][j]) continue;
        PointSet &A = m_sets[i];
#pragma omp parallel for schedule(static)
        for (long long a = 0; a < (long long)A.m_n; a++)
          query(g, m_sets[j], A.point((unsigned int)a), i == j ? (long long)a : -1, A.m_neighbors[j][a]);
      }
    }
  }
  // neighbours of one point of a set in every active set
  void find_neighbors(unsigned int point_set_id, unsigned int point_index,
                      std::vector<std::vector<unsigned int>> &neighbors) {
    const std::size_t ns = m_sets.size();
    neighbors.assign(ns, std::vector<unsigned int>());
    for (std::size_t j = 0; j < ns; j++) {
      if (!m_active[point_set_id][j] || m_sets[j].m_n == 0) continue;
      Grid g;
      build_grid(m_sets[j], g);
      query(g, m_sets[j], m_sets[point_set_id].point(point_index), j == point_set_id ? (long long)point_index : -1,
            neighbors[j]);
    }
  }

 private:
  struct Grid {
    std::unordered_map<int64_t, std::vector<unsigned int>> cells;
  };
  static int64_t key(int64_t x, int64_t y, int64_t z) {
    return ((x + (1 << 20)) << 42) | ((y + (1 << 20)) << 21) | (z + (1 << 20));
  }
  // cells slightly wider than r, so that a rounding error in a cell coordinate cannot hide a
  // pair closer than r
  int64_t cell_of(Real v) const { return (int64_t)std::floor(v / (m_r * Real(1.0001))); }
  void build_grid(const PointSet &S, Grid &g) const {
    for (unsigned int b = 0; b < S.m_n; b++) {
      const Real *p = S.point(b);
      g.cells[key(cell_of(p[0]), cell_of(p[1]), cell_of(p[2]))].push_back(b);
    }
  }
  void query(const Grid &g, const PointSet &S, const Real *pa, long long self, std::vector<unsigned int> &out) const {
    const Real r2 = m_r * m_r;
    const int64_t cx = cell_of(pa[0]), cy = cell_of(pa[1]), cz = cell_of(pa[2]);
    out.clear();
    for (int64_t dz = -1; dz <= 1; dz++)
      for (int64_t dy = -1; dy <= 1; dy++)
        for (int64_t dx = -1; dx <= 1; dx++) {
          auto it = g.cells.find(key(cx + dx, cy + dy, cz + dz));
          if (it == g.cells.end()) continue;
          for (unsigned int b : it->second) {
            if ((long long)b == self) continue;
            const Real *pb = S.point(b);
            const Real ex = pa[0] - pb[0], ey = pa[1] - pb[1], ez = pa[2] - pb[2];
            if (((ex * ex + ey * ey) + ez * ez) < r2) out.push_back(b);
          }
        }
    std::sort(out.begin(), out.end());
  }

  Real m_r;
  std::vector<PointSet> m_sets;
  std::vector<std::vector<unsigned char>> m_active;
};

}  // namespace CompactNSearch
