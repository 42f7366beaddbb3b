// ref_sampling.cpp — runs the reference's own RegularTriangleSampling::sampleMesh
// (SPlisHSPlasH/Utilities/RegularTriangleSampling.cpp, compiled with it by oracle/build_ref.sh)
// on a mesh read from a file and writes the samples. Test infrastructure only
// (tests/golden/make_golden.py).
// Input (float64): n_vertices, n_faces, max_distance, vertices[n][3], faces[m][3].
// Output (float64): the samples, [k][3].
#include <cstdio>
#include <vector>

#include "SPlisHSPlasH/Utilities/RegularTriangleSampling.h"

int main(int argc, char **argv) {
  if (argc != 3) return 2;
  std::vector<double> d;
  FILE *f = fopen(argv[1], "rb");
  if (!f) return 2;
  double x;
  while (fread(&x, sizeof(double), 1, f) == 1) d.push_back(x);
  fclose(f);
  const unsigned int nv = (unsigned int)d[0], nf = (unsigned int)d[1];
  const Real dist = (Real)d[2];
  std::vector<Vector3r> v(nv);
  for (unsigned int i = 0; i < nv; i++) v[i] = Vector3r((Real)d[3 + 3 * i], (Real)d[4 + 3 * i], (Real)d[5 + 3 * i]);
  std::vector<unsigned int> faces(3 * nf);
  for (unsigned int i = 0; i < 3 * nf; i++) faces[i] = (unsigned int)d[3 + 3 * nv + i];
  std::vector<Vector3r> samples;
  SPH::RegularTriangleSampling::sampleMesh(nv, v.data(), nf, faces.data(), dist, samples);
  FILE *o = fopen(argv[2], "wb");
  if (!o) return 2;
  for (const auto &p : samples)
    for (int c = 0; c < 3; c++) {
      const double y = (double)p[c];
      fwrite(&y, sizeof(double), 1, o);
    }
  fclose(o);
  return 0;
}
