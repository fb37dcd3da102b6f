// Test helper (built by tests/test_tile_plan.py against the in-tree library):
// reads a cell list (int64 n, then n x 6 doubles x0 x1 y0 y1 z0 z1), builds the
// assembly tile plan and checks it: every cell exactly once; tiles of at most 8
// runs (1 or 2 across x) and 64 levels; at every level a cell's z0 is the z1 of
// the cell above in its run, its y0 the y1 of the cell before it in y (same x
// extent and levels), and in a 2-wide tile its x0 the x1 of the cell before it
// in x (same y extent and levels).  Prints the shares of cells that take a face
// over in z, y and x; exit status 0 when the plan holds.
#include <cstdint>
#include <cstdio>
#include <set>
#include <vector>

namespace grada {
void build_tile_plan(const double *prisms, int64_t n_cells, std::vector<int32_t> &tiles,
                     std::vector<int64_t> &cells);
}

int main(int argc, char **argv) {
  if (argc != 2) return 2;
  FILE *f = std::fopen(argv[1], "rb");
  if (!f) return 3;
  int64_t n = 0;
  if (std::fread(&n, 8, 1, f) != 1) return 3;
  std::vector<double> p(6 * (size_t)n);
  if (std::fread(p.data(), 8, p.size(), f) != p.size()) return 3;
  std::fclose(f);
  std::vector<int32_t> t;
  std::vector<int64_t> c;
  grada::build_tile_plan(p.data(), n, t, c);
  std::set<int64_t> seen;
  int64_t bad = 0, sz = 0, sy = 0, sx = 0;
  const int64_t n_tiles = (int64_t)t.size() / 4;
  for (int64_t i = 0; i < n_tiles; i++) {
    const int off = t[4 * i], runs = t[4 * i + 1], levels = t[4 * i + 2];
    const int nx = t[4 * i + 3] > 1 ? 2 : 1;
    if (runs < 1 || runs > 8 || runs % nx || levels < 1 || levels > 64) bad++;
    for (int a = 0; a < runs; a++)
      for (int k = 0; k < levels; k++) {
        const int64_t cell = c[off + (int64_t)a * levels + k];
        if (cell < 0 || cell >= n || !seen.insert(cell).second) {
          bad++;
          continue;
        }
        const double *u = &p[6 * cell];
        const int x = a % nx, y = a / nx;
        if (k > 0) {
          const double *v = &p[6 * c[off + (int64_t)a * levels + k - 1]];
          if (u[0] == v[0] && u[1] == v[1] && u[2] == v[2] && u[3] == v[3] && u[4] == v[5]) sz++;
          else bad++;
        }
        if (y > 0) {
          const double *v = &p[6 * c[off + (int64_t)(a - nx) * levels + k]];
          if (u[0] == v[0] && u[1] == v[1] && u[2] == v[3] && u[4] == v[4] && u[5] == v[5]) sy++;
          else bad++;
        }
        if (x > 0) {
          const double *v = &p[6 * c[off + (int64_t)(a - 1) * levels + k]];
          if (u[0] == v[1] && u[2] == v[2] && u[3] == v[3] && u[4] == v[4] && u[5] == v[5]) sx++;
          else bad++;
        }
      }
  }
  std::printf("cells %lld tiles %lld bad %lld zshare %.4f yshare %.4f xshare %.4f\n", (long long)n,
              (long long)n_tiles, (long long)bad, (double)sz / n, (double)sy / n, (double)sx / n);
  return (bad == 0 && (int64_t)seen.size() == n) ? 0 : 1;
}
