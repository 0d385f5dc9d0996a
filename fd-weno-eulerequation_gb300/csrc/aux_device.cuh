// Device bodies shared by the per-solve kernels (aux_kernels.cu) and the
// persistent batched kernel (batch_kernel.cuh): the boundary fill of one
// ghost entry and a node's wave-speed sum for the time step.
#pragma once

#include "convert.cuh"
#include "guard.cuh"
#include "wenofd_internal.h"

namespace wenofd {
namespace dev {

// Member owning work item `item` of a batch's prefix array (n+1 entries).
// The prefix arrays and the member table are read-only for the whole launch.
__device__ __forceinline__ int owner(const int *prefix, int n, int item) {
  int lo = 0, hi = n;  // prefix[lo] <= item < prefix[hi]
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (__ldg(&prefix[mid]) <= item) lo = mid;
    else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ long long at(const Geom &g, int r, int ei, int ej) {
  return WENOFD_IXC(g.guard, unsigned(r) < 4u && unsigned(ei) < unsigned(g.nxt) && unsigned(ej) < unsigned(g.pitch),
                    r * g.plane + (long long)ei * g.pitch + ej, 4 * g.plane);
}

// exchangeGhostCellsValue (src/WENOFD.cpp:850-929, one rank) + setBoundary
// (998-1159).  Every ghost node a stencil reads -- x ghosts on interior
// rows, y ghosts on interior columns -- is a function of interior nodes
// only, so all of them are filled in one pass:
//   x, periodic  : ghost[sx-k] = U[ex-1-k], ghost[ex-1+k] = U[sx+k]
//                  (node-based: the duplicated end node is skipped)
//   SYMMETRIC    : mirror about the boundary node, ghost[sx-k] = U[sx+k]
//   SLIP         : mirror and negate the normal momentum
//   SPECIAL      : initial-condition value at the boundary node (table)
// The y direction uses the bottom condition on both sides (line 1009).
// Corner ghosts (x ghost and y ghost at once) are never read by the sweeps
// (lines 513-797) but are read by the indicator's 5x5 windows; they get the
// reference's values: its y fill runs over every column, ghost columns
// included, after the x exchange, and its x conditions then run over every
// row, ghost rows included.  So a corner is the y rule applied to the
// x-periodic source column (x periodic) or the x rule applied to the y ghost
// of the interior source column (x not periodic).
// Number of ghost entries (each covers the 4 conserved variables).
__host__ __device__ __forceinline__ int bc_entries(const Geom &g) { return 8 * g.nx + 8 * g.ny + 64; }

// Ghost entry t in [0, bc_entries(g)).  Reads go through L2 only: in the
// persistent batched kernel the sources were written by other blocks.
__device__ __forceinline__ void bc_fill_entry(const Geom &g, double *U, const double *special, const int t) {
  const int nxg = 4 * g.nx, nyg = 4 * g.ny;
  const int sx = kGhost, ex = kGhost + g.nx, sy = kGhost, ey = kGhost + g.ny;
  {
    if (t < 2 * nyg) {  // x ghosts on interior rows
      const int side = t / nyg, rem = t - side * nyg;
      const int e1 = rem / g.ny + 1, ej = sy + (rem - (e1 - 1) * g.ny);
      const int bc = side == 0 ? g.bc_left : g.bc_right;
      const int dst = side == 0 ? sx - e1 : ex - 1 + e1;
      int src;
      if (bc == kPeriod) src = side == 0 ? ex - 1 - e1 : sx + e1;
      else src = side == 0 ? sx + e1 : ex - 1 - e1;
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        double v;
        if (bc == kSpecial) v = special[WENOFD_SPECIAL(g, 8 * g.nxt + (side * 4 + r) * g.nyt + ej)];
        else v = __ldcg(&U[at(g, r, src, ej)]);
        if (bc == kSlip && r == 1) v *= -1;
        U[at(g, r, dst, ej)] = v;
      }
    } else if (t >= 2 * nyg + 2 * nxg) {  // the 4 x 16 corner ghosts
      const int c = t - 2 * nyg - 2 * nxg;
      const int sidex = c >> 5, sidey = (c >> 4) & 1;
      const int kx = ((c >> 2) & 3) + 1, ky = (c & 3) + 1;
      const int ei = sidex == 0 ? sx - kx : ex - 1 + kx;
      const int ej = sidey == 0 ? sy - ky : ey - 1 + ky;
      const int bcx = sidex == 0 ? g.bc_left : g.bc_right;
      const int srcy = g.bc_y == kPeriod ? (sidey == 0 ? ey - 1 - ky : sy + ky) : (sidey == 0 ? sy + ky : ey - 1 - ky);
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        double v;
        if (bcx == kSpecial) {
          v = special[WENOFD_SPECIAL(g, 8 * g.nxt + (sidex * 4 + r) * g.nyt + ej)];
        } else {
          const int col = bcx == kPeriod ? (sidex == 0 ? ex - 1 - kx : sx + kx) : (sidex == 0 ? sx + kx : ex - 1 - kx);
          // y rule at ghost column ei (x periodic: its interior rows hold
          // column col) or at interior column col (x not periodic)
          if (g.bc_y == kSpecial) v = special[WENOFD_SPECIAL(g, (sidey * 4 + r) * g.nxt + (bcx == kPeriod ? ei : col))];
          else v = __ldcg(&U[at(g, r, col, srcy)]);
          if (g.bc_y == kSlip && r == 2) v *= -1;
          if (bcx == kSlip && r == 1) v *= -1;
        }
        U[at(g, r, ei, ej)] = v;
      }
    } else {  // y ghosts on interior columns
      const int u = t - 2 * nyg;
      const int side = u / nxg, rem = u - side * nxg;
      const int e1 = rem / g.nx + 1, ei = sx + (rem - (e1 - 1) * g.nx);
      const int bc = g.bc_y;
      const int dst = side == 0 ? sy - e1 : ey - 1 + e1;
      int src;
      if (bc == kPeriod) src = side == 0 ? ey - 1 - e1 : sy + e1;
      else src = side == 0 ? sy + e1 : ey - 1 - e1;
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        double v;
        if (bc == kSpecial) v = special[WENOFD_SPECIAL(g, (side * 4 + r) * g.nxt + ei)];
        else v = __ldcg(&U[at(g, r, ei, src)]);
        if (bc == kSlip && r == 2) v *= -1;
        U[at(g, r, ei, dst)] = v;
      }
    }
  }
}

// A node's s depends only on its four state values.  In uniform regions
// (the quadrants of a Riemann problem) every node ties for the maximum and
// the FP64 evaluation (five divisions and a square root on a pipe at 1/73 of
// the FP32 rate) would run for each of them: a thread skips a node whose
// values are bit for bit those of the last node it evaluated, which leaves
// the maximum and the NaN flag unchanged.
struct SpeedMemo {
  long long k[4] = {0, 0, 0, 0};
  bool valid = false;
  __device__ __forceinline__ bool repeat(double rho, double mu, double mv, double E) {
    const long long a = __double_as_longlong(rho), b = __double_as_longlong(mu), c = __double_as_longlong(mv),
                    d = __double_as_longlong(E);
    const bool same = valid && a == k[0] && b == k[1] && c == k[2] && d == k[3];
    k[0] = a;
    k[1] = b;
    k[2] = c;
    k[3] = d;
    valid = true;
    return same;
  }
};

// One node's s = lx/dx + ly/dy exactly as calculateDeltaT forms it
// (src/WENOFD.cpp:419-423 with utils/equations.hpp:137-147).
__device__ __forceinline__ double exact_speed(const Geom &g, double rho, double mu, double mv, double E) {
  const double gamma = g.gamma;
  const double u = mu / rho, v = mv / rho;
  const double p = (gamma - 1.0) * (E - 0.5 * rho * (u * u + v * v));
  const double cs = sqrt(gamma * p / rho);
  const double lx = fabs(u * 1.0 + v * 0.0) + cs;
  const double ly = fabs(u * 0.0 + v * 1.0) + cs;
  return lx / g.dx + ly / g.dy;
}

// FP32 estimate s32 of a node's s and a bound e with |s32 - s| <= e.  Error
// budget (eps = 2^-23): inputs truncated to FP32 (eps each), u and v from
// __fdividef (3 eps), kinetic energy ke (< 9.5 eps relative), so
// p = (gamma-1)(E - ke) carries at most 12 eps (|E| + ke) / (E - ke)
// relative error (the cancellation term); c = sqrt(gamma p / rho) half of
// that plus 2 eps; the final bound takes 4x the propagated sum.  Nodes with
// a non-positive or non-finite FP32 pressure get e = inf.
__device__ __forceinline__ void screen_speed(const Geom &g, double rho_d, double mu_d, double mv_d, double E_d,
                                             float &s, float &e) {
  // Explicit round-to-nearest operations: no multiply-add contraction, so
  // every translation unit (the stage kernels' fused screen, the reduction
  // kernels, the batched kernel) computes the same s and e.
  const float eps = 1.1920929e-07f;
  const float r = f64_to_f32(rho_d), mu = f64_to_f32(mu_d), mv = f64_to_f32(mv_d), E = f64_to_f32(E_d);
  const float u = __fdividef(mu, r), v = __fdividef(mv, r);
  const float ke = __fmul_rn(__fmul_rn(0.5f, r), __fadd_rn(__fmul_rn(u, u), __fmul_rn(v, v)));
  const float pp = __fsub_rn(E, ke);
  const float c2 = __fdividef(__fmul_rn(g.gamma32, __fmul_rn(__fsub_rn(g.gamma32, 1.0f), pp)), r);
  if (!(pp > 0.0f) || !(c2 > 0.0f) || !(c2 < 3.0e38f) || !(fabsf(u) < 3.0e38f) || !(fabsf(v) < 3.0e38f)) {
    s = 0.0f;
    e = __int_as_float(0x7f800000);
    return;
  }
  const float c = __fsqrt_rn(c2);
  const float au = fabsf(u), av = fabsf(v);
  s = __fadd_rn(__fmul_rn(__fadd_rn(au, c), g.inv_dx32), __fmul_rn(__fadd_rn(av, c), g.inv_dy32));
  const float rp = __fdiv_rn(__fmul_rn(__fmul_rn(12.0f, eps), __fadd_rn(fabsf(E), ke)), pp);
  const float rc = __fadd_rn(__fmul_rn(0.5f, rp), __fmul_rn(2.0f, eps));
  const float ex = __fadd_rn(__fmul_rn(__fmul_rn(au, 3.0f), eps), __fmul_rn(c, rc));
  const float ey = __fadd_rn(__fmul_rn(__fmul_rn(av, 3.0f), eps), __fmul_rn(c, rc));
  e = __fadd_rn(__fmul_rn(4.0f, __fadd_rn(__fadd_rn(__fmul_rn(ex, g.inv_dx32), __fmul_rn(ey, g.inv_dy32)),
                                          __fmul_rn(__fmul_rn(s, 4.0f), eps))),
                __fmul_rn(1e-12f, s));
}


}  // namespace dev
}  // namespace wenofd
