// Host build of the fixed-point collision (lbm_fx.cuh) on a periodic lattice:
// reads f[nx][ny][9] (float64, reference layout), runs `steps` steps of
// collide (fx::collide_q, float64 BGK for nodes outside its range) + periodic
// streaming on the stored deviations, writes f back.  Test infrastructure for
// tests/test_fx_host.py; compile with -ffp-contract=off.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "../../lattice_boltzmann_parallel_solver_gb300/csrc/lbm_fx.cuh"

using namespace lbm;
static const int CX[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1}, CY[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1};
static const double W[9] = {4.0 / 9, 1.0 / 9, 1.0 / 9, 1.0 / 9, 1.0 / 9, 1.0 / 36, 1.0 / 36, 1.0 / 36, 1.0 / 36};

static void collide_double(double f[9], double omega) {
  const double rho = ((f[0] + f[1]) + (f[2] + f[3])) + ((f[4] + f[5]) + (f[6] + f[7])) + f[8];
  const double ux = ((f[1] + f[5] + f[8]) - (f[3] + f[6] + f[7])) / rho;
  const double uy = ((f[2] + f[5] + f[6]) - (f[4] + f[7] + f[8])) / rho;
  const double usq = ux * ux + uy * uy;
  for (int i = 0; i < 9; ++i) {
    const double cu = CX[i] * ux + CY[i] * uy;
    f[i] += (W[i] * rho * (1 + 3 * cu + 4.5 * cu * cu - 1.5 * usq) - f[i]) * omega;
  }
}

int main(int argc, char** argv) {
  if (argc != 7) return 2;
  const int nx = atoi(argv[1]), ny = atoi(argv[2]), steps = atoi(argv[3]);
  const double omega = atof(argv[4]);
  const size_t n = (size_t)nx * ny * 9;
  std::vector<double> f(n);
  FILE* in = fopen(argv[5], "rb");
  if (!in || fread(f.data(), 8, n, in) != n) return 3;
  fclose(in);
  std::vector<int64_t> d(n), post(n);
  for (size_t k = 0; k < n; ++k) d[k] = fx::to_fx(f[k], W[k % 9]);
  const fx::QConsts c = fx::q_consts(omega);
  long fallback = 0;
  for (int s = 0; s < steps; ++s) {
    for (size_t b = 0; b < n; b += 9) {
      int64_t g[9];
      for (int i = 0; i < 9; ++i) g[i] = d[b + i];
      if (!fx::collide_q(g, c)) {
        double h[9];
        for (int i = 0; i < 9; ++i) h[i] = fx::from_fx(g[i], W[i]);
        collide_double(h, omega);
        for (int i = 0; i < 9; ++i) g[i] = fx::to_fx(h[i], W[i]);
        ++fallback;
      }
      for (int i = 0; i < 9; ++i) post[b + i] = g[i];
    }
    for (int x = 0; x < nx; ++x)
      for (int y = 0; y < ny; ++y)
        for (int i = 0; i < 9; ++i) {
          const int xs = (x - CX[i] + nx) % nx, ys = (y - CY[i] + ny) % ny;
          d[((size_t)x * ny + y) * 9 + i] = post[((size_t)xs * ny + ys) * 9 + i];
        }
  }
  for (size_t k = 0; k < n; ++k) f[k] = fx::from_fx(d[k], W[k % 9]);
  FILE* out = fopen(argv[6], "wb");
  if (!out || fwrite(f.data(), 8, n, out) != n) return 4;
  fclose(out);
  printf("%ld\n", fallback);
  return 0;
}
