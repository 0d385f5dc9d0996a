#include "cases.h"

#include <cmath>
#include <cstring>
#include <stdexcept>

namespace wenofd {

uint64_t splitmix64(uint64_t &state) {
  uint64_t z = (state += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

double uniform01(uint64_t &state) { return double(splitmix64(state) >> 11) * (1.0 / 9007199254740992.0); }

CaseSpec make_case(int testcase, uint64_t seed) {
  CaseSpec c;
  c.testcase = testcase;
  c.seed = seed;
  switch (testcase) {
    case 0:  // SMOOTH, utils/equations.hpp:404-442
      c.xl = 0.0; c.xr = 2.0; c.yl = 0.0; c.yr = 2.0; c.t_end = 1.0;
      c.exact = 1;
      break;
    case 1: {  // Riemann1, utils/equations.hpp:443-521
      const double q[16] = {0.8, 0.0, 0.0, 1.0, 1.0, 0.7276, 0.0, 1.0, 1.0, 0.0, 0.7276, 1.0, 0.5313, 0.0, 0.0, 0.4};
      c.xl = 0.0; c.xr = 2.0; c.yl = 0.0; c.yr = 2.0; c.t_end = 0.52;
      c.bc_left = c.bc_right = c.bc_bottom = c.bc_top = 3;
      std::memcpy(c.quad, q, sizeof(q));
      c.interface = 1.0;
      break;
    }
    case 2: {  // Riemann2, utils/equations.hpp:522-600
      const double q[16] = {0.138, 1.206, 1.206, 0.029, 0.5323, 1.206, 0.0, 0.3,
                            0.5323, 0.0, 1.206, 0.3, 1.5, 0.0, 0.0, 1.5};
      c.xl = 0.0; c.xr = 1.0; c.yl = 0.0; c.yr = 1.0; c.t_end = 0.8;
      c.bc_left = c.bc_right = c.bc_bottom = c.bc_top = 3;
      std::memcpy(c.quad, q, sizeof(q));
      break;
    }
    case 3:  // RTI, utils/equations.hpp:601-642
      c.xl = 0.0; c.xr = 0.25; c.yl = 0.0; c.yr = 1.0; c.t_end = 1.95;
      c.bc_left = c.bc_right = 1;
      c.bc_bottom = c.bc_top = 2;
      c.gamma = 5.0 / 3.0;
      c.gravity = 1;
      break;
    case 4: {  // four-quadrant Riemann problem with seeded states, interface (0.8, 0.8)
      uint64_t s = seed;
      c.xl = 0.0; c.xr = 1.0; c.yl = 0.0; c.yr = 1.0; c.t_end = 0.3;
      c.bc_left = c.bc_right = c.bc_bottom = c.bc_top = 3;
      for (int k = 0; k < 4; ++k) {
        c.quad[4 * k + 0] = 0.1 + (1.5 - 0.1) * uniform01(s);
        c.quad[4 * k + 1] = -1.2 + (1.2 - -1.2) * uniform01(s);
        c.quad[4 * k + 2] = -1.2 + (1.2 - -1.2) * uniform01(s);
        c.quad[4 * k + 3] = 0.03 + (1.5 - 0.03) * uniform01(s);
      }
      break;
    }
    case 5:  // periodic shear layer on [0,1]^2
      c.xl = 0.0; c.xr = 1.0; c.yl = 0.0; c.yr = 1.0; c.t_end = 1.0;
      break;
    default:
      throw std::invalid_argument("Invalid example number");
  }
  return c;
}

double node_x(const CaseSpec &c, double dx, int ei) {
  const double proc_left = c.xl + 0 * dx;
  const double ghost_left = proc_left - dx * 4;
  return ghost_left + ei * dx;
}

double node_y(const CaseSpec &c, double dy, int ej) {
  const double ghost_low = c.yl - dy * 4;
  return ghost_low + ej * dy;
}

namespace {
// getU0, utils/equations.hpp:649-662
void prim_to_cons(double gamma, double rho, double u, double v, double pre, double U[4]) {
  const double E = pre / (gamma - 1.0) + 0.5 * rho * (u * u + v * v);
  U[0] = rho;
  U[1] = rho * u;
  U[2] = rho * v;
  U[3] = E;
}
}  // namespace

void u0(const CaseSpec &c, double x, double y, double U[4]) {
  switch (c.testcase) {
    case 0:
      prim_to_cons(c.gamma, 1 + 0.2 * std::sin(M_PI * (x + y)), 0.7, 0.3, 1, U);
      return;
    case 1:
    case 2:
    case 4: {
      const double s = c.interface;
      const int k = (x < s) ? (y < s ? 0 : 1) : (y < s ? 2 : 3);
      prim_to_cons(c.gamma, c.quad[4 * k], c.quad[4 * k + 1], c.quad[4 * k + 2], c.quad[4 * k + 3], U);
      return;
    }
    case 3: {
      const double rho = (y <= 0.5) ? 2.0 : 1.0;
      const double pre = (y <= 0.5) ? 1 + 2 * y : y + 1.5;
      const double cs = std::sqrt(c.gamma * pre / rho);
      const double v = -0.025 * cs * std::cos(8 * M_PI * x);
      prim_to_cons(c.gamma, rho, 0, v, pre, U);
      return;
    }
    case 5: {
      const bool inside = std::fabs(y - 0.5) < 0.25;
      prim_to_cons(c.gamma, inside ? 2.0 : 1.0, inside ? 0.5 : -0.5, 0.01 * std::sin(4 * M_PI * x), 2.5, U);
      return;
    }
  }
  throw std::invalid_argument("Invalid example number");
}

// The shear layer adds N(0, 1e-3) noise to v, drawn by Box-Muller from the
// splitmix64 stream of (seed ^ 0x5DEECE66D) on the nx-1 by ny-1 distinct
// nodes in ei-major order; the periodic duplicate nodes (last row / column)
// copy node 0 of their line so both copies of a periodic node agree.
void initial_state(const CaseSpec &c, int nx, int ny, double dx, double dy, double *out) {
  const size_t plane = size_t(nx) * ny;
  uint64_t s = c.seed ^ 0x5DEECE66DULL;
  for (int i = 0; i < nx; ++i)
    for (int j = 0; j < ny; ++j) {
      double q[4];
      if (c.testcase == 5) {
        const int si = (i == nx - 1) ? 0 : i, sj = (j == ny - 1) ? 0 : j;
        if (si != i || sj != j) {
          for (int r = 0; r < 4; ++r) q[r] = out[r * plane + size_t(si) * ny + sj];
        } else {
          const double x = node_x(c, dx, i + 4), y = node_y(c, dy, j + 4);
          const bool inside = std::fabs(y - 0.5) < 0.25;
          const double u1 = 1.0 - uniform01(s);
          const double u2 = uniform01(s);
          const double noise = 1e-3 * (std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * M_PI * u2));
          const double v = 0.01 * std::sin(4 * M_PI * x) + noise;
          prim_to_cons(c.gamma, inside ? 2.0 : 1.0, inside ? 0.5 : -0.5, v, 2.5, q);
        }
      } else {
        u0(c, node_x(c, dx, i + 4), node_y(c, dy, j + 4), q);
      }
      for (int r = 0; r < 4; ++r) out[r * plane + size_t(i) * ny + j] = q[r];
    }
}

std::vector<double> special_table(const CaseSpec &c, int nx, int ny, double dx, double dy) {
  const int nxt = nx + 8, nyt = ny + 8;
  std::vector<double> tab(8 * size_t(nxt) + 8 * size_t(nyt), 0.0);
  const bool any = c.bc_left == 2 || c.bc_right == 2 || c.bc_bottom == 2;
  if (!any) return tab;
  double q[4];
  for (int ei = 0; ei < nxt; ++ei) {
    u0(c, node_x(c, dx, ei), node_y(c, dy, 4), q);
    for (int r = 0; r < 4; ++r) tab[r * nxt + ei] = q[r];
    u0(c, node_x(c, dx, ei), node_y(c, dy, ny + 3), q);
    for (int r = 0; r < 4; ++r) tab[4 * nxt + r * nxt + ei] = q[r];
  }
  for (int ej = 0; ej < nyt; ++ej) {
    u0(c, node_x(c, dx, 4), node_y(c, dy, ej), q);
    for (int r = 0; r < 4; ++r) tab[8 * nxt + r * nyt + ej] = q[r];
    u0(c, node_x(c, dx, nx + 4), node_y(c, dy, ej), q);
    for (int r = 0; r < 4; ++r) tab[8 * nxt + 4 * nyt + r * nyt + ej] = q[r];
  }
  return tab;
}

}  // namespace wenofd
