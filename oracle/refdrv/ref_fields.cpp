// Fixture driver (test infrastructure, built only in the oracle's _ref/ tree
// from the reference sources): evaluates the reference's own prism kernels,
// GravFormula::field_caused_by_single_prism, for every (observation, cell)
// pair the way Fwd::compute_G does (src/Forward_modelling/Fwd.cpp:47-78).
//
// Usage: ref_fields <in.bin> <out.bin>
//   in.bin : int64 n_cells, int64 n_obs, uint32 mask,
//            n_cells*6 doubles (x0 x1 y0 y1 z0 z1), n_obs*3 doubles (x y z)
//   out.bin: G column-major, (n_fields*n_obs) x n_cells doubles
#include <bitset>
#include <cstdint>
#include <cstdio>
#include <vector>

#include "GravFormula.h"
#include "Point.h"
#include "RectPrism.h"

int main(int argc, char **argv) {
  if (argc != 3) {
    std::fprintf(stderr, "usage: %s in.bin out.bin\n", argv[0]);
    return 2;
  }
  FILE *f = std::fopen(argv[1], "rb");
  if (!f) return 3;
  int64_t nc = 0, no = 0;
  uint32_t mask = 0;
  if (std::fread(&nc, 8, 1, f) != 1 || std::fread(&no, 8, 1, f) != 1 ||
      std::fread(&mask, 4, 1, f) != 1)
    return 4;
  std::vector<double> pr(6 * nc), ob(3 * no);
  if (std::fread(pr.data(), 8, pr.size(), f) != pr.size() ||
      std::fread(ob.data(), 8, ob.size(), f) != ob.size())
    return 5;
  std::fclose(f);
  std::bitset<10> flag(mask);
  std::vector<int> idx;
  for (int b = 0; b < 10; b++)
    if (flag[b]) idx.push_back(b);
  const int64_t nf = (int64_t)idx.size();
  const int64_t nd = nf * no;
  std::vector<double> G((size_t)(nd * nc));
  for (int64_t i = 0; i < no; i++) {
    Point p(ob[3 * i], ob[3 * i + 1], ob[3 * i + 2]);
#pragma omp parallel for
    for (int64_t j = 0; j < nc; j++) {
      const double *q = &pr[6 * j];
      RectPrism rect(q[0], q[2], q[4], q[1], q[3], q[5]);
      GravFormula gra;
      std::vector<double> field;
      gra.field_caused_by_single_prism(p, rect, 1.0, field, flag);
      for (int64_t k = 0; k < nf; k++) G[(size_t)((i + k * no) + j * nd)] = field[idx[k]];
    }
  }
  FILE *o = std::fopen(argv[2], "wb");
  if (!o) return 6;
  std::fwrite(G.data(), 8, G.size(), o);
  std::fclose(o);
  return 0;
}
