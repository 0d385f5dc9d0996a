/*
 * wenofd_oracle.c — CPU restatement of the reference's per-step hot path.
 *
 * TEST INFRASTRUCTURE, NOT PRODUCT: the checker for the CUDA path.  Only
 * tests/, the smoke() check and bench.py's CPU-baseline leg may load it.
 *
 * Every function restates one reference function, operation by operation in
 * the reference's evaluation order, so that with -ffp-contract=off it rounds
 * exactly like the reference built with -ffp-contract=off.  Citations are to
 * files of infinity-07/FD-WENO-EulerEquation.
 */
#include "wenofd_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* include/Utility.hpp:5-11 */
static const double C1_3 = 1.0 / 3.0;
static const double C1_4 = 1.0 / 4.0;
static const double C1_6 = 1.0 / 6.0;
static const double C5_6 = 5.0 / 6.0;
static const double C7_6 = 7.0 / 6.0;
static const double C11_6 = 11.0 / 6.0;
static const double C13_12 = 13.0 / 12.0;

#define NXT(g) ((g)->nx + 2 * ORC_NG)
#define NYT(g) ((g)->ny + 2 * ORC_NG)
#define AT(g, A, r, i, j) (A)[((size_t)(r) * NXT(g) + (size_t)(i)) * NYT(g) + (size_t)(j)]

/* ------------------------------------------------------------------ WENO */

/* WENO5threconstruction, include/Utility.hpp:415-456 (WENO-JS, eps 1e-6). */
static double weno5_js(double a, double b, double c, double d, double e) {
  const double d0 = 0.1, d1 = 0.6, d2 = 0.3;
  double t1 = (a - 2 * b + c);
  double t2 = (a - 4 * b + 3 * c);
  const double beta0 = 13.0 / 12.0 * t1 * t1 + 0.25 * t2 * t2;
  t1 = (b - 2 * c + d);
  t2 = (b - d);
  const double beta1 = 13.0 / 12.0 * t1 * t1 + 0.25 * t2 * t2;
  t1 = (c - 2 * d + e);
  t2 = (3 * c - 4 * d + e);
  const double beta2 = 13.0 / 12.0 * t1 * t1 + 0.25 * t2 * t2;
  const double eps = 1.0e-6;
  double w0 = d0 / ((eps + beta0) * (eps + beta0));
  double w1 = d1 / ((eps + beta1) * (eps + beta1));
  double w2 = d2 / ((eps + beta2) * (eps + beta2));
  const double sum = w0 + w1 + w2;
  w0 = w0 / sum;
  w1 = w1 / sum;
  w2 = w2 / sum;
  const double h0 = 1.0 / 3.0 * a - 7.0 / 6.0 * b + 11.0 / 6.0 * c;
  const double h1 = -1.0 / 6 * b + 5.0 / 6.0 * c + 1.0 / 3.0 * d;
  const double h2 = 1.0 / 3.0 * c + 5.0 / 6.0 * d - 1.0 / 6.0 * e;
  return w0 * h0 + w1 * h1 + w2 * h2;
}

/* WENO5Zthreconstruction, include/Utility.hpp:457-504 (WENO-Z, eps 1e-20).
 * The weight products are evaluated left to right, tau*inv*tau*inv, as in
 * the reference (lines 489-491). */
static void wenoz_core(double a, double b, double c, double d, double e, double w[3], double p[3]) {
  double t1, t2;
  t1 = (a - 2.0 * b + c);
  t2 = (a - 4.0 * b + 3.0 * c);
  const double betam = C13_12 * t1 * t1 + C1_4 * t2 * t2;
  t1 = (b - 2.0 * c + d);
  t2 = (b - d);
  const double beta = C13_12 * t1 * t1 + C1_4 * t2 * t2;
  t1 = (c - 2.0 * d + e);
  t2 = (3.0 * c - 4.0 * d + e);
  const double betap = C13_12 * t1 * t1 + C1_4 * t2 * t2;
  const double eps = 1.0e-20;
  const double inv_betam = 1.0 / (betam + eps);
  const double inv_beta = 1.0 / (beta + eps);
  const double inv_betap = 1.0 / (betap + eps);
  const double d0 = 0.1, d1 = 0.6, d2 = 0.3;
  const double tau = fabs(betam - betap);
  double w0 = d0 * (1.0 + (tau * inv_betam * tau * inv_betam));
  double w1 = d1 * (1.0 + (tau * inv_beta * tau * inv_beta));
  double w2 = d2 * (1.0 + (tau * inv_betap * tau * inv_betap));
  const double ws = w0 + w1 + w2;
  w0 /= ws;
  w1 /= ws;
  w2 /= ws;
  w[0] = w0;
  w[1] = w1;
  w[2] = w2;
  p[0] = C1_3 * a - C7_6 * b + C11_6 * c;
  p[1] = -C1_6 * b + C5_6 * c + C1_3 * d;
  p[2] = C1_3 * c + C5_6 * d - C1_6 * e;
}

static double weno5_z(double a, double b, double c, double d, double e) {
  double w[3], p[3];
  wenoz_core(a, b, c, d, e, w, p);
  return w[0] * p[0] + w[1] * p[1] + w[2] * p[2];
}

/* WENO5ZPtheconstruction, include/Utility.hpp:505-558.  lambda = pow(dx, 2/3)
 * is passed in (the reference computes it per call from m_deltaX, also in
 * the y sweep: src/WENOFD.cpp:836). */
static double weno5_zp(double a, double b, double c, double d, double e, double lambda) {
  double t1, t2;
  t1 = (a - 2 * b + c);
  t2 = (a - 4 * b + 3 * c);
  const double betam = 13.0 / 12.0 * t1 * t1 + 0.25 * t2 * t2;
  t1 = (b - 2 * c + d);
  t2 = (b - d);
  const double beta = 13.0 / 12.0 * t1 * t1 + 0.25 * t2 * t2;
  t1 = (c - 2 * d + e);
  t2 = (3 * c - 4 * d + e);
  const double betap = 13.0 / 12.0 * t1 * t1 + 0.25 * t2 * t2;
  const double tau = fabs(betam - betap);
  const double d0 = 0.1, d1 = 0.6, d2 = 0.3;
  const double eps = 1.0e-40;
  double w0 = d0 * (1 + pow((tau + eps) / (betam + eps), 2) + lambda * (betam + eps) / (tau + eps));
  double w1 = d1 * (1 + pow((tau + eps) / (beta + eps), 2) + lambda * (beta + eps) / (tau + eps));
  double w2 = d2 * (1 + pow((tau + eps) / (betap + eps), 2) + lambda * (betap + eps) / (tau + eps));
  const double sum = w0 + w1 + w2;
  w0 = w0 / sum;
  w1 = w1 / sum;
  w2 = w2 / sum;
  const double p0 = 1.0 / 3.0 * a - 7.0 / 6.0 * b + 11.0 / 6.0 * c;
  const double p1 = -1.0 / 6 * b + 5.0 / 6.0 * c + 1.0 / 3.0 * d;
  const double p2 = 1.0 / 3.0 * c + 5.0 / 6.0 * d - 1.0 / 6.0 * e;
  return w0 * p0 + w1 * p1 + w2 * p2;
}

/* WENO5ZPItheconstruction, include/Utility.hpp:559-615. */
static double weno5_zpi(double a, double b, double c, double d, double e) {
  double t1, t2;
  t1 = (a - 2 * b + c);
  t2 = (a - 4 * b + 3 * c);
  const double betam = 13.0 / 12.0 * t1 * t1 + 0.25 * t2 * t2;
  t1 = (b - 2 * c + d);
  t2 = (b - d);
  const double beta = 13.0 / 12.0 * t1 * t1 + 0.25 * t2 * t2;
  t1 = (c - 2 * d + e);
  t2 = (3 * c - 4 * d + e);
  const double betap = 13.0 / 12.0 * t1 * t1 + 0.25 * t2 * t2;
  const double tau = fabs(betam - betap);
  const double lambda = 3.3;
  /* std::max(a, b) is (a < b) ? b : a; std::min(a, b) is (b < a) ? b : a */
  const double mx_in = (beta < betap) ? betap : beta;
  const double betaMAX = (betam < mx_in) ? mx_in : betam;
  const double mn_in = (betap < beta) ? betap : beta;
  const double betaMIN = (mn_in < betam) ? mn_in : betam;
  const double alpha = 1 - (betaMIN / (betaMAX + 1e-40));
  const double d0 = 0.1, d1 = 0.6, d2 = 0.3;
  const double eps = 1.0e-40;
  double w0 = d0 * (1 + pow(tau / (betam + eps), 2) + lambda * alpha * (betam) / (betaMAX + eps));
  double w1 = d1 * (1 + pow(tau / (beta + eps), 2) + lambda * alpha * (beta) / (betaMAX + eps));
  double w2 = d2 * (1 + pow(tau / (betap + eps), 2) + lambda * alpha * (betap) / (betaMAX + eps));
  const double sum = w0 + w1 + w2;
  w0 = w0 / sum;
  w1 = w1 / sum;
  w2 = w2 / sum;
  const double p0 = 1.0 / 3.0 * a - 7.0 / 6.0 * b + 11.0 / 6.0 * c;
  const double p1 = -1.0 / 6 * b + 5.0 / 6.0 * c + 1.0 / 3.0 * d;
  const double p2 = 1.0 / 3.0 * c + 5.0 / 6.0 * d - 1.0 / 6.0 * e;
  return w0 * p0 + w1 * p1 + w2 * p2;
}

/* CWENOFD::useWENO dispatch, src/WENOFD.cpp:823-848. */
double orc_weno5(int scheme, double a, double b, double c, double d, double e, double zp_lambda) {
  switch (scheme) {
    case ORC_WENOJS: return weno5_js(a, b, c, d, e);
    case ORC_WENOZ: return weno5_z(a, b, c, d, e);
    case ORC_WENOZP: return weno5_zp(a, b, c, d, e, zp_lambda);
    case ORC_WENOZPI: return weno5_zpi(a, b, c, d, e);
  }
  return NAN;
}

void orc_wenoz_weights(double a, double b, double c, double d, double e, double w[3]) {
  double p[3];
  wenoz_core(a, b, c, d, e, w, p);
}

/* --------------------------------------------------------------- physics */

/* getPhyFluxX / getPhyFluxY, utils/equations.hpp:105-134. dir 0 = x. */
void orc_phys_flux(int dir, double gamma, const double U[4], double F[4]) {
  const double rho = U[0];
  const double u = U[1] / U[0];
  const double v = U[2] / U[0];
  const double E = U[3];
  const double p = (gamma - 1.0) * (E - 0.5 * rho * (u * u + v * v));
  if (dir == 0) {
    F[0] = rho * u;
    F[1] = rho * u * u + p;
    F[2] = rho * u * v;
    F[3] = (E + p) * u;
  } else {
    F[0] = rho * v;
    F[1] = rho * u * v;
    F[2] = rho * v * v + p;
    F[3] = (E + p) * v;
  }
}

/* getMaxEigenValueX / Y, utils/equations.hpp:149-171. */
double orc_max_eig(int dir, double gamma, const double U[4]) {
  const double rho = U[0];
  const double u = U[1] / U[0];
  const double v = U[2] / U[0];
  const double E = U[3];
  const double p = (gamma - 1.0) * (E - 0.5 * rho * (u * u + v * v));
  const double c = sqrt(gamma * p / rho);
  return (dir == 0 ? fabs(u) : fabs(v)) + c;
}

/* getMaxEigenValue(U, nx, ny), utils/equations.hpp:137-147: the form
 * calculateDeltaT calls with (1, 0) and (0, 1). */
static double max_eig_n(double gamma, const double U[4], double nx, double ny) {
  const double rho = U[0];
  const double u = U[1] / U[0];
  const double v = U[2] / U[0];
  const double E = U[3];
  const double p = (gamma - 1.0) * (E - 0.5 * rho * (u * u + v * v));
  const double c = sqrt(gamma * p / rho);
  return fabs(u * nx + v * ny) + c;
}

/* fluxSplitX / fluxSplitY, utils/equations.hpp:365-393: pointwise
 * Lax-Friedrichs splitting with alpha = |u|+c (or |v|+c). */
void orc_flux_split(int dir, double gamma, const double U[4], double fm[4], double fp[4]) {
  double F[4];
  orc_phys_flux(dir, gamma, U, F);
  const double ws = orc_max_eig(dir, gamma, U);
  for (int r = 0; r != 4; ++r) {
    fm[r] = 0.5 * (F[r] - ws * U[r]);
    fp[r] = 0.5 * (F[r] + ws * U[r]);
  }
}

/* getLEigenMatrixX/Y (utils/equations.hpp:174-236) and getREigenMatrixX/Y
 * (239-299).  L and R are row-major 4x4: M[row*4+col] = eigMatrix[row][col]. */
void orc_eigen_lr(int dir, double gamma, const double U[4], double L[16], double R[16]) {
  const double rho = U[0];
  const double u = U[1] / U[0];
  const double v = U[2] / U[0];
  const double E = U[3];
  const double p = (gamma - 1.0) * (E - 0.5 * rho * (u * u + v * v));
  const double c = sqrt(gamma * p / rho);
  const double B1 = (gamma - 1) / (c * c);
  const double B2 = B1 * (u * u + v * v) / 2;
  const double H = (E + p) / rho;
  if (dir == 0) {
    L[0] = (B2 + u / c) / 2;          L[1] = -(B1 * u + 1.0 / c) / 2;  L[2] = -(B1 * v) / 2; L[3] = B1 / 2;
    L[4] = v;                         L[5] = 0;                        L[6] = -1;            L[7] = 0;
    L[8] = (1 - B2);                  L[9] = B1 * u;                   L[10] = B1 * v;       L[11] = -B1;
    L[12] = (B2 - u / c) / 2;         L[13] = -(B1 * u - 1.0 / c) / 2; L[14] = -B1 * v / 2; L[15] = B1 / 2;

    R[0] = 1;          R[1] = 0;   R[2] = 1;                   R[3] = 1;
    R[4] = u - c;      R[5] = 0;   R[6] = u;                   R[7] = u + c;
    R[8] = v;          R[9] = -1;  R[10] = v;                  R[11] = v;
    R[12] = H - c * u; R[13] = -v; R[14] = (u * u + v * v) / 2; R[15] = H + c * u;
  } else {
    L[0] = (B2 + v / c) / 2;  L[1] = -(B1 * u) / 2; L[2] = -(B1 * v + 1.0 / c) / 2;  L[3] = B1 / 2;
    L[4] = -u;                L[5] = 1;             L[6] = 0;                        L[7] = 0;
    L[8] = 1 - B2;            L[9] = B1 * u;        L[10] = B1 * v;                  L[11] = -B1;
    L[12] = (B2 - v / c) / 2; L[13] = -(B1 * u) / 2; L[14] = -(B1 * v - 1.0 / c) / 2; L[15] = B1 / 2;

    R[0] = 1;          R[1] = 0;  R[2] = 1;                   R[3] = 1;
    R[4] = u;          R[5] = 1;  R[6] = u;                   R[7] = u;
    R[8] = v - c;      R[9] = 0;  R[10] = v;                  R[11] = v + c;
    R[12] = H - c * v; R[13] = u; R[14] = (u * u + v * v) / 2; R[15] = H + c * v;
  }
}

/* ----------------------------------------------------------------- cases */

unsigned long long orc_splitmix64(unsigned long long *state) {
  unsigned long long z = (*state += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

double orc_uniform01(unsigned long long *state) {
  return (double)(orc_splitmix64(state) >> 11) * (1.0 / 9007199254740992.0);
}

/* setEquationParameters, utils/equations.hpp:400-646, plus the two seeded
 * cases (four-quadrant Riemann problem with states drawn from the seed, and
 * the periodic shear layer). */
void orc_case_setup(int testcase, unsigned long long seed, orc_case *c) {
  memset(c, 0, sizeof(*c));
  c->testcase = testcase;
  c->seed = seed;
  c->gamma = 1.4;
  c->interface = 0.8;
  switch (testcase) {
    case ORC_SMOOTH:
      c->xl = 0.0; c->xr = 2.0; c->yl = 0.0; c->yr = 2.0; c->t_end = 1.0;
      c->bc_left = c->bc_right = c->bc_top = c->bc_bottom = ORC_PERIOD;
      c->exact = 1;
      break;
    case ORC_RIEMANN1: {
      static const double q[16] = {0.8, 0.0, 0.0, 1.0, 1.0, 0.7276, 0.0, 1.0,
                                   1.0, 0.0, 0.7276, 1.0, 0.5313, 0.0, 0.0, 0.4};
      c->xl = 0.0; c->xr = 2.0; c->yl = 0.0; c->yr = 2.0; c->t_end = 0.52;
      c->bc_left = c->bc_right = c->bc_top = c->bc_bottom = ORC_SYMMETRIC;
      memcpy(c->quad, q, sizeof(q));
      c->interface = 1.0;
      break;
    }
    case ORC_RIEMANN2: {
      static const double q[16] = {0.138, 1.206, 1.206, 0.029, 0.5323, 1.206, 0.0, 0.3,
                                   0.5323, 0.0, 1.206, 0.3, 1.5, 0.0, 0.0, 1.5};
      c->xl = 0.0; c->xr = 1.0; c->yl = 0.0; c->yr = 1.0; c->t_end = 0.8;
      c->bc_left = c->bc_right = c->bc_top = c->bc_bottom = ORC_SYMMETRIC;
      memcpy(c->quad, q, sizeof(q));
      break;
    }
    case ORC_RTI:
      c->xl = 0.0; c->xr = 0.25; c->yl = 0.0; c->yr = 1.0; c->t_end = 1.95;
      c->bc_left = c->bc_right = ORC_SLIP;
      c->bc_top = c->bc_bottom = ORC_SPECIAL;
      c->gamma = 5.0 / 3.0;
      c->gravity = 1;
      break;
    case ORC_RIEMANN_SEEDED: {
      unsigned long long s = seed;
      c->xl = 0.0; c->xr = 1.0; c->yl = 0.0; c->yr = 1.0; c->t_end = 0.3;
      c->bc_left = c->bc_right = c->bc_top = c->bc_bottom = ORC_SYMMETRIC;
      for (int k = 0; k < 4; ++k) {
        c->quad[4 * k + 0] = 0.1 + (1.5 - 0.1) * orc_uniform01(&s);
        c->quad[4 * k + 1] = -1.2 + (1.2 - -1.2) * orc_uniform01(&s);
        c->quad[4 * k + 2] = -1.2 + (1.2 - -1.2) * orc_uniform01(&s);
        c->quad[4 * k + 3] = 0.03 + (1.5 - 0.03) * orc_uniform01(&s);
      }
      break;
    }
    case ORC_SHEAR:
      c->xl = 0.0; c->xr = 1.0; c->yl = 0.0; c->yr = 1.0; c->t_end = 1.0;
      c->bc_left = c->bc_right = c->bc_top = c->bc_bottom = ORC_PERIOD;
      break;
  }
}

/* src/WENOFD.cpp:73-80: node spacing over ELEMNUM-1 intervals; ghost-origin
 * coordinate xl - dx*4, node ei at origin + ei*dx (line 100). */
void orc_grid_setup(const orc_case *c, int nx, int ny, int scheme, orc_grid *g) {
  memset(g, 0, sizeof(*g));
  g->nx = nx;
  g->ny = ny;
  g->scheme = scheme;
  g->bc_left = c->bc_left;
  g->bc_right = c->bc_right;
  g->bc_bottom = c->bc_bottom;
  g->bc_top = c->bc_top;
  g->gravity = c->gravity;
  g->gamma = c->gamma;
  g->dx = (c->xr - c->xl) / (nx - 1);
  g->dy = (c->yr - c->yl) / (ny - 1);
  g->zp_lambda = pow(g->dx, 2.0 / 3.0);
  g->xl = c->xl;
  g->yl = c->yl;
  g->special = NULL;
}

double orc_node_x(const orc_grid *g, int ei) {
  const double proc_left = g->xl + 0 * g->dx;
  const double ghost_left = proc_left - g->dx * ORC_NG;
  return ghost_left + ei * g->dx;
}

double orc_node_y(const orc_grid *g, int ej) {
  const double ghost_low = g->yl - g->dy * ORC_NG;
  return ghost_low + ej * g->dy;
}

static void prim_to_cons(double gamma, double rho, double u, double v, double pre, double U[4]) {
  /* getU0, utils/equations.hpp:649-662 */
  const double E = pre / (gamma - 1.0) + 0.5 * rho * (u * u + v * v);
  U[0] = rho;
  U[1] = rho * u;
  U[2] = rho * v;
  U[3] = E;
}

/* The initial-condition lambdas of setEquationParameters. */
void orc_u0(const orc_case *c, double x, double y, double U[4]) {
  switch (c->testcase) {
    case ORC_SMOOTH:
      prim_to_cons(c->gamma, 1 + 0.2 * sin(M_PI * (x + y)), 0.7, 0.3, 1, U);
      return;
    case ORC_RIEMANN1:
    case ORC_RIEMANN2:
    case ORC_RIEMANN_SEEDED: {
      const double s = c->interface;
      const int k = (x < s) ? (y < s ? 0 : 1) : (y < s ? 2 : 3);
      prim_to_cons(c->gamma, c->quad[4 * k], c->quad[4 * k + 1], c->quad[4 * k + 2], c->quad[4 * k + 3], U);
      return;
    }
    case ORC_RTI: {
      const double rho = (y <= 0.5) ? 2.0 : 1.0;
      const double pre = (y <= 0.5) ? 1 + 2 * y : y + 1.5;
      const double cs = sqrt(c->gamma * pre / rho);
      const double v = -0.025 * cs * cos(8 * M_PI * x);
      prim_to_cons(c->gamma, rho, 0, v, pre, U);
      return;
    }
    case ORC_SHEAR: {
      const double inside = fabs(y - 0.5) < 0.25;
      prim_to_cons(c->gamma, inside ? 2.0 : 1.0, inside ? 0.5 : -0.5, 0.01 * sin(4 * M_PI * x), 2.5, U);
      return;
    }
  }
  U[0] = U[1] = U[2] = U[3] = NAN;
}

/* initializeAve, src/WENOFD.cpp:165-188, for the reference's cases.  The
 * shear layer adds N(0, 1e-3) noise to v, drawn (Box-Muller) on the NX-1 x
 * NY-1 distinct nodes in ei-major order; the duplicate periodic end nodes
 * (ei = NX-1, ej = NY-1) copy node 0 so the periodic state is consistent. */
void orc_initial_state(const orc_case *c, const orc_grid *g, double *U) {
  const size_t n = (size_t)4 * NXT(g) * NYT(g);
  memset(U, 0, n * sizeof(double));
  unsigned long long s = c->seed ^ 0x5DEECE66DULL;
  for (int i = 0; i < g->nx; ++i) {
    for (int j = 0; j < g->ny; ++j) {
      const int ei = i + ORC_NG, ej = j + ORC_NG;
      double q[4];
      if (c->testcase == ORC_SHEAR) {
        const int si = (i == g->nx - 1) ? 0 : i, sj = (j == g->ny - 1) ? 0 : j;
        if (si != i || sj != j) {
          for (int r = 0; r < 4; ++r) q[r] = AT(g, U, r, si + ORC_NG, sj + ORC_NG);
        } else {
          const double x = orc_node_x(g, ei), y = orc_node_y(g, ej);
          const double inside = fabs(y - 0.5) < 0.25;
          const double u1 = 1.0 - orc_uniform01(&s);
          const double u2 = orc_uniform01(&s);
          const double noise = 1e-3 * (sqrt(-2.0 * log(u1)) * cos(2.0 * M_PI * u2));
          const double v = 0.01 * sin(4 * M_PI * x) + noise;
          prim_to_cons(c->gamma, inside ? 2.0 : 1.0, inside ? 0.5 : -0.5, v, 2.5, q);
        }
      } else {
        orc_u0(c, orc_node_x(g, ei), orc_node_y(g, ej), q);
      }
      for (int r = 0; r < 4; ++r) AT(g, U, r, ei, ej) = q[r];
    }
  }
}

/* SPECIAL boundary values (src/WENOFD.cpp:1045-1058, 1092-1102, 1138-1149)
 * are getU0 at fixed nodes, so they are tabulated once:
 *   [0, 4*NXT)            bottom, r-major, per ei: U0 at node (ei, startY)
 *   [4*NXT, 8*NXT)        top,    per ei: U0 at node (ei, endY-1)
 *   [8*NXT, 8*NXT+4*NYT)  left,   per ej: U0 at node (startX, ej)
 *   [.., 8*NXT+8*NYT)     right,  per ej: U0 at node (endX, ej), the first
 *                         ghost column, as the reference does (line 1144). */
long orc_special_table_size(const orc_grid *g) { return 8L * NXT(g) + 8L * NYT(g); }

void orc_special_table(const orc_case *c, const orc_grid *g, double *tab) {
  const int nxt = NXT(g), nyt = NYT(g);
  const int sx = ORC_NG, ex = ORC_NG + g->nx, sy = ORC_NG, ey = ORC_NG + g->ny;
  double q[4];
  for (int ei = 0; ei < nxt; ++ei) {
    orc_u0(c, orc_node_x(g, ei), orc_node_y(g, sy), q);
    for (int r = 0; r < 4; ++r) tab[r * nxt + ei] = q[r];
    orc_u0(c, orc_node_x(g, ei), orc_node_y(g, ey - 1), q);
    for (int r = 0; r < 4; ++r) tab[4 * nxt + r * nxt + ei] = q[r];
  }
  for (int ej = 0; ej < nyt; ++ej) {
    orc_u0(c, orc_node_x(g, sx), orc_node_y(g, ej), q);
    for (int r = 0; r < 4; ++r) tab[8 * nxt + r * nyt + ej] = q[r];
    orc_u0(c, orc_node_x(g, ex), orc_node_y(g, ej), q);
    for (int r = 0; r < 4; ++r) tab[8 * nxt + 4 * nyt + r * nyt + ej] = q[r];
  }
}

/* -------------------------------------------------------------- boundary */

/* exchangeGhostCellsValue with one rank (src/WENOFD.cpp:850-929) followed
 * by setBoundary (998-1159).  The exchange always runs and makes x periodic
 * on the interior rows, skipping the duplicated end node:
 * ghost[startX-k] = U[endX-1-k], ghost[endX-1+k] = U[startX+k], k = 1..4.
 * setBoundary then fills y over every column with the BOTTOM condition for
 * both sides (line 1009), then x over every row for non-periodic sides. */
void orc_fill_boundary(const orc_grid *g, double *U) {
  const int sx = ORC_NG, ex = ORC_NG + g->nx, sy = ORC_NG, ey = ORC_NG + g->ny;
  for (int k = 1; k <= ORC_NG; ++k)
    for (int ej = sy; ej < ey; ++ej)
      for (int r = 0; r < 4; ++r) {
        AT(g, U, r, sx - k, ej) = AT(g, U, r, ex - 1 - k, ej);
        AT(g, U, r, ex - 1 + k, ej) = AT(g, U, r, sx + k, ej);
      }
  orc_fill_boundary_slab(g, U, 1, 1);
}

/* setBoundary of one rank's x-slab (src/WENOFD.cpp:998-1159) after its x
 * ghost columns of the interior rows were exchanged: the y conditions over
 * every column, ghost columns included, then the x conditions on the sides
 * that are domain edges (left_edge: rank 0, right_edge: the last rank) over
 * every row.  On a slab grid g->nx is the slab's node count and the SPECIAL
 * table is the slab's slice (y part [8][slab nx + 8], x part as global). */
void orc_fill_boundary_slab(const orc_grid *g, double *U, int left_edge, int right_edge) {
  const int nxt = NXT(g), nyt = NYT(g);
  const int sx = ORC_NG, ex = ORC_NG + g->nx, sy = ORC_NG, ey = ORC_NG + g->ny;
  for (int ei = 0; ei != nxt; ei++) {
    for (int e1 = 1; e1 <= ORC_NG; ++e1) {
      switch (g->bc_bottom) {
        case ORC_PERIOD:
          for (int r = 0; r != 4; ++r) {
            AT(g, U, r, ei, sy - e1) = AT(g, U, r, ei, ey - 1 - e1);
            AT(g, U, r, ei, ey - 1 + e1) = AT(g, U, r, ei, sy + e1);
          }
          break;
        case ORC_SYMMETRIC:
        case ORC_SLIP:
          for (int r = 0; r != 4; ++r) {
            AT(g, U, r, ei, sy - e1) = AT(g, U, r, ei, sy + e1);
            AT(g, U, r, ei, ey - 1 + e1) = AT(g, U, r, ei, ey - 1 - e1);
          }
          if (g->bc_bottom == ORC_SLIP) {
            AT(g, U, 2, ei, sy - e1) *= -1;
            AT(g, U, 2, ei, ey - 1 + e1) *= -1;
          }
          break;
        case ORC_SPECIAL:
          for (int r = 0; r != 4; ++r) {
            AT(g, U, r, ei, sy - e1) = g->special[r * nxt + ei];
            AT(g, U, r, ei, ey - 1 + e1) = g->special[4 * nxt + r * nxt + ei];
          }
          break;
      }
    }
  }
  for (int ej = 0; ej != nyt && left_edge; ej++) {
    for (int e1 = 1; e1 <= ORC_NG; ++e1) {
      switch (g->bc_left) {
        case ORC_SYMMETRIC:
        case ORC_SLIP:
          for (int r = 0; r != 4; ++r) AT(g, U, r, sx - e1, ej) = AT(g, U, r, sx + e1, ej);
          if (g->bc_left == ORC_SLIP) AT(g, U, 1, sx - e1, ej) *= -1;
          break;
        case ORC_SPECIAL:
          for (int r = 0; r != 4; ++r) AT(g, U, r, sx - e1, ej) = g->special[8 * nxt + r * nyt + ej];
          break;
        default:
          break;
      }
    }
  }
  for (int ej = 0; ej != nyt && right_edge; ej++) {
    for (int e1 = 1; e1 <= ORC_NG; ++e1) {
      switch (g->bc_right) {
        case ORC_SYMMETRIC:
        case ORC_SLIP:
          for (int r = 0; r != 4; ++r) AT(g, U, r, ex - 1 + e1, ej) = AT(g, U, r, ex - 1 - e1, ej);
          if (g->bc_right == ORC_SLIP) AT(g, U, 1, ex - 1 + e1, ej) *= -1;
          break;
        case ORC_SPECIAL:
          for (int r = 0; r != 4; ++r)
            AT(g, U, r, ex - 1 + e1, ej) = g->special[8 * nxt + 4 * nyt + r * nyt + ej];
          break;
        default:
          break;
      }
    }
  }
}

/* ------------------------------------------------------------ RHS sweeps */

/* One face of a characteristic WENO sweep, src/WENOFD.cpp:526-643 (x) and
 * 668-791 (y): average state, eigenvectors, projection of five F+ (nodes
 * face-3..face+1) and five F- (face-2..face+2) with sums in index order,
 * WENO per characteristic field (minus side mirrored), back-projection. */
static void face_flux(const orc_grid *g, int dir, const double Um[4], const double U0[4],
                      double fp[][4], double fm[][4], double out[4]) {
  double ave[4], L[16], R[16], vp[5][4], vm[5][4], vh[4];
  for (int r = 0; r != 4; r++) ave[r] = 0.5 * (Um[r] + U0[r]);
  orc_eigen_lr(dir, g->gamma, ave, L, R);
  for (int s = 0; s < 5; ++s) {
    for (int k = 0; k < 4; ++k) {
      double a = L[k * 4 + 0] * fp[s][0];
      a += L[k * 4 + 1] * fp[s][1];
      a += L[k * 4 + 2] * fp[s][2];
      a += L[k * 4 + 3] * fp[s][3];
      vp[s][k] = a;
      double b = L[k * 4 + 0] * fm[s + 1][0];
      b += L[k * 4 + 1] * fm[s + 1][1];
      b += L[k * 4 + 2] * fm[s + 1][2];
      b += L[k * 4 + 3] * fm[s + 1][3];
      vm[s][k] = b;
    }
  }
  for (int k = 0; k < 4; ++k) {
    const double hp = orc_weno5(g->scheme, vp[0][k], vp[1][k], vp[2][k], vp[3][k], vp[4][k], g->zp_lambda);
    const double hm = orc_weno5(g->scheme, vm[4][k], vm[3][k], vm[2][k], vm[1][k], vm[0][k], g->zp_lambda);
    vh[k] = hp + hm;
  }
  for (int r = 0; r < 4; ++r) {
    double f = R[r * 4 + 0] * vh[0];
    f += R[r * 4 + 1] * vh[1];
    f += R[r * 4 + 2] * vh[2];
    f += R[r * 4 + 3] * vh[3];
    out[r] = f;
  }
}

/* assembleRHS (src/WENOFD.cpp:454-465) = zero + assembleBoundaryTerm
 * (481-798) + assembleSourceTerm (800-821).  Fills U's ghosts; rhs is a full
 * array whose interior is written. */
void orc_assemble_rhs(const orc_grid *g, double *U, double *rhs) {
  orc_fill_boundary(g, U);
  orc_assemble_rhs_ghosted(g, U, rhs);
}

/* The same with U's ghosts already filled (an x-slab after its exchange and
 * orc_fill_boundary_slab). */
void orc_assemble_rhs_ghosted(const orc_grid *g, const double *U, double *rhs) {
  const int nxt = NXT(g), nyt = NYT(g);
  const int sx = ORC_NG, ex = ORC_NG + g->nx, sy = ORC_NG, ey = ORC_NG + g->ny;
  for (int r = 0; r < 4; ++r)
    for (int ei = sx; ei < ex; ++ei)
      for (int ej = sy; ej < ey; ++ej) AT(g, rhs, r, ei, ej) = 0.0;

  const int nmax = nxt > nyt ? nxt : nyt;
  /* Lines are independent, so they are spread over threads; each face is
   * still computed by one thread in the reference's operation order. */
#pragma omp parallel
  {
    double(*fp)[4] = malloc(sizeof(double[4]) * nmax);
    double(*fm)[4] = malloc(sizeof(double[4]) * nmax);
    double(*face)[4] = malloc(sizeof(double[4]) * (nmax + 1));
    double q[4], qm[4];
#pragma omp for schedule(static)
    for (int ej = sy; ej < ey; ej++) { /* x sweep, lines 512-649 */
      for (int ei = 0; ei != nxt; ei++) {
        for (int r = 0; r < 4; ++r) q[r] = AT(g, U, r, ei, ej);
        orc_flux_split(0, g->gamma, q, fm[ei], fp[ei]);
      }
      for (int f = sx; f != ex + 1; f++) {
        for (int r = 0; r < 4; ++r) {
          qm[r] = AT(g, U, r, f - 1, ej);
          q[r] = AT(g, U, r, f, ej);
        }
        face_flux(g, 0, qm, q, &fp[f - 3], &fm[f - 3], face[f]);
      }
      for (int ei = sx; ei != ex; ei++)
        for (int r = 0; r != 4; ++r) AT(g, rhs, r, ei, ej) += -(face[ei + 1][r] - face[ei][r]) / g->dx;
    }
#pragma omp for schedule(static)
    for (int ei = sx; ei < ex; ei++) { /* y sweep, lines 651-797 */
      for (int ej = 0; ej != nyt; ej++) {
        for (int r = 0; r < 4; ++r) q[r] = AT(g, U, r, ei, ej);
        orc_flux_split(1, g->gamma, q, fm[ej], fp[ej]);
      }
      for (int f = sy; f != ey + 1; ++f) {
        for (int r = 0; r < 4; ++r) {
          qm[r] = AT(g, U, r, ei, f - 1);
          q[r] = AT(g, U, r, ei, f);
        }
        face_flux(g, 1, qm, q, &fp[f - 3], &fm[f - 3], face[f]);
      }
      for (int ej = sy; ej != ey; ej++)
        for (int r = 0; r != 4; ++r) AT(g, rhs, r, ei, ej) += -(face[ej + 1][r] - face[ej][r]) / g->dy;
    }
    free(fp);
    free(fm);
    free(face);
  }

  if (g->gravity) { /* RTI source, g = 1 */
    const double g_g0 = 1.0;
    for (int ei = sx; ei != ex; ei++)
      for (int ej = sy; ej != ey; ej++) {
        AT(g, rhs, 3, ei, ej) += AT(g, U, 2, ei, ej) * g_g0;
        AT(g, rhs, 2, ei, ej) += AT(g, U, 0, ei, ej) * g_g0;
      }
  }
}

/* calculateDeltaT, src/WENOFD.cpp:398-452, including its update rule
 * (a NaN candidate replaces the running value and is itself replaced by the
 * next candidate).  Returns 1 when the final step is NaN (the reference
 * aborts there). */
int orc_calc_dt(const orc_grid *g, const double *U, double cfl, double now, double t_end, double *dt) {
  double timestep = 1.0;
  const int sx = ORC_NG, ex = ORC_NG + g->nx, sy = ORC_NG, ey = ORC_NG + g->ny;
  double q[4];
  for (int ei = sx; ei != ex; ei++)
    for (int ej = sy; ej != ey; ej++) {
      for (int r = 0; r != 4; ++r) q[r] = AT(g, U, r, ei, ej);
      const double ex_ = max_eig_n(g->gamma, q, 1, 0);
      const double ey_ = max_eig_n(g->gamma, q, 0, 1);
      const double tmp = cfl / (ex_ / g->dx + ey_ / g->dy);
      if (tmp > timestep)
        continue;
      else
        timestep = tmp;
    }
  if (t_end - now < timestep) timestep = t_end - now;
  *dt = timestep;
  return timestep != timestep;
}

/* RunRK1 / RunRK2 / RunRK3, src/WENOFD.cpp:301-396.  rk: 0, 1, 2. */
void orc_rk_step(const orc_grid *g, int rk, double *U, double *Un, double *rhs, double dt) {
  const int sx = ORC_NG, ex = ORC_NG + g->nx, sy = ORC_NG, ey = ORC_NG + g->ny;
  if (rk == 0) {
    orc_assemble_rhs(g, U, rhs);
    for (int ei = sx; ei != ex; ei++)
      for (int ej = sy; ej != ey; ej++)
        for (int r = 0; r < 4; r++) AT(g, U, r, ei, ej) += dt * AT(g, rhs, r, ei, ej);
    return;
  }
  static const double A2[2][3] = {{1.0, 0.0, 1.0}, {0.5, 0.5, 0.5}};
  static const double A3[3][3] = {{1.0, 0.0, 1.0}, {3.0 / 4.0, 1.0 / 4.0, 1.0 / 4.0}, {1.0 / 3.0, 2.0 / 3.0, 2.0 / 3.0}};
  for (int ei = sx; ei != ex; ei++)
    for (int ej = sy; ej != ey; ej++)
      for (int r = 0; r != 4; ++r) AT(g, Un, r, ei, ej) = AT(g, U, r, ei, ej);
  const int nst = rk == 1 ? 2 : 3;
  for (int st = 0; st != nst; st++) {
    orc_assemble_rhs(g, U, rhs);
    const double a = rk == 1 ? A2[st][0] : A3[st][0];
    const double b = rk == 1 ? A2[st][1] : A3[st][1];
    const double c = rk == 1 ? A2[st][2] : A3[st][2];
    for (int ei = sx; ei != ex; ei++)
      for (int ej = sy; ej != ey; ej++)
        for (int r = 0; r < 4; r++)
          AT(g, U, r, ei, ej) = a * AT(g, Un, r, ei, ej) + b * AT(g, U, r, ei, ej) + c * dt * AT(g, rhs, r, ei, ej);
  }
}

/* The time loop of CWENOFD::run, src/WENOFD.cpp:213-239, optionally capped
 * at max_steps (< 0: no cap).  Returns 1 on a NaN step. */
int orc_run(const orc_grid *g, int rk, double cfl, double *U, double *Un, double *rhs, double *now,
            double t_end, long max_steps, long *steps, double *dts, long dts_cap) {
  long count = 0;
  while (fabs(*now - t_end) > 1e-9) {
    if (max_steps >= 0 && count >= max_steps) break;
    double dt;
    if (orc_calc_dt(g, U, cfl, *now, t_end, &dt)) {
      *steps = count;
      return 1;
    }
    orc_rk_step(g, rk, U, Un, rhs, dt);
    *now += dt;
    if (dts && count < dts_cap) dts[count] = dt;
    count++;
  }
  *steps = count;
  return 0;
}

/* outputAccuracy, src/WENOFD.cpp:1308-1382, for the smooth case's exact
 * density 1 + 0.2 sin(pi (x + y - t)) (utils/equations.hpp:438-439).
 * out = {Linf, L1, L2}; L1/L2 normalised by NX*NY. */
void orc_error_norms(const orc_grid *g, const double *U, double t, double out[3]) {
  const int sx = ORC_NG, ex = ORC_NG + g->nx, sy = ORC_NG, ey = ORC_NG + g->ny;
  double e1 = 0, e2 = 0, einf = 0;
  for (int ei = sx; ei != ex; ei++)
    for (int ej = sy; ej != ey; ej++) {
      const double x = orc_node_x(g, ei), y = orc_node_y(g, ej);
      const double uref = 1 + 0.2 * sin(M_PI * (x + y - t));
      const double err = fabs(uref - AT(g, U, 0, ei, ej));
      e1 += err;
      e2 += pow(err, 2);
      if (err > einf) einf = err;
    }
  out[0] = einf;
  out[1] = e1 / g->nx / g->ny;
  out[2] = sqrt(e2 / g->nx / g->ny);
}

/* Interior sums of the conserved variables (total mass, momenta, energy). */
void orc_conservation_sums(const orc_grid *g, const double *U, double out[4]) {
  for (int r = 0; r < 4; ++r) {
    double s = 0;
    for (int ei = ORC_NG; ei < ORC_NG + g->nx; ++ei)
      for (int ej = ORC_NG; ej < ORC_NG + g->ny; ++ej) s += AT(g, U, r, ei, ej);
    out[r] = s;
  }
}

/* ------------------------------------------- learned indicator (own spec) */

static float feat_pressure(float gamma, const float q[4]) {
  const float u = q[1] / q[0], v = q[2] / q[0];
  return (gamma - 1.0f) * (q[3] - 0.5f * q[0] * (u * u + v * v));
}

static void normalise_window(const float w[25], float out[25]) {
  const float c = w[12];
  float R = 0.0f;
  for (int k = 0; k < 25; ++k) {
    const float d = fabsf(w[k] - c);
    if (d > R) R = d;
  }
  if (R <= 1e-4f * (fabsf(c) + 1e-12f)) {
    for (int k = 0; k < 25; ++k) out[k] = 0.0f;
    return;
  }
  const float inv = 1.0f / R;
  for (int k = 0; k < 25; ++k) out[k] = (w[k] - c) * inv;
}

void orc_cell_features(const orc_grid *g, const double *U, float *features) {
  const float gam = (float)g->gamma;
  for (int i = 0; i < g->nx; ++i)
    for (int j = 0; j < g->ny; ++j) {
      float wr[25], wp[25];
      for (int a = 0; a < 5; ++a)
        for (int b = 0; b < 5; ++b) {
          float q[4];
          for (int r = 0; r < 4; ++r) q[r] = (float)AT(g, U, r, ORC_NG + i + a - 2, ORC_NG + j + b - 2);
          wr[a * 5 + b] = q[0];
          wp[a * 5 + b] = feat_pressure(gam, q);
        }
      float *o = features + ((size_t)i * g->ny + j) * 50;
      normalise_window(wr, o);
      normalise_window(wp, o + 25);
    }
}

/* max |w_k - d_k| of WENO-Z for one characteristic field and side; 0 when
 * the stencil's range is <= 1e-2 of `scale` (the largest characteristic
 * magnitude at the face): such a stencil changes the flux negligibly
 * whatever its weights. */
static double face_side_deviation(const double v[5], double scale) {
  double lo = v[0], hi = v[0];
  for (int s = 1; s < 5; ++s) {
    if (v[s] < lo) lo = v[s];
    if (v[s] > hi) hi = v[s];
  }
  if (hi - lo <= 1e-2 * scale) return 0.0;
  double w[3];
  orc_wenoz_weights(v[0], v[1], v[2], v[3], v[4], w);
  const double d[3] = {0.1, 0.6, 0.3};
  double dev = 0.0;
  for (int k = 0; k < 3; ++k)
    if (fabs(w[k] - d[k]) > dev) dev = fabs(w[k] - d[k]);
  return dev;
}

/* Face between nodes (ei-1, ej) and (ei, ej) (dir 0) or (ei, ej-1) and
 * (ei, ej) (dir 1), full-array indices. */
static double face_deviation(const orc_grid *g, const double *U, int dir, int ei, int ej) {
  const int di = dir == 0 ? 1 : 0, dj = dir == 0 ? 0 : 1;
  double um[4], u0[4], ave[4], L[16], R[16], fp[6][4], fm[6][4];
  for (int r = 0; r < 4; ++r) {
    um[r] = AT(g, U, r, ei - di, ej - dj);
    u0[r] = AT(g, U, r, ei, ej);
    ave[r] = 0.5 * (um[r] + u0[r]);
  }
  orc_eigen_lr(dir, g->gamma, ave, L, R);
  for (int s = 0; s < 6; ++s) { /* nodes face-3 .. face+2 */
    double q[4];
    for (int r = 0; r < 4; ++r) q[r] = AT(g, U, r, ei + (s - 3) * di, ej + (s - 3) * dj);
    orc_flux_split(dir, g->gamma, q, fm[s], fp[s]);
  }
  double vp[4][5], vm[4][5], scale = 0.0;
  for (int k = 0; k < 4; ++k)
    for (int s = 0; s < 5; ++s) {
      vp[k][s] = L[k * 4 + 0] * fp[s][0] + L[k * 4 + 1] * fp[s][1] + L[k * 4 + 2] * fp[s][2] + L[k * 4 + 3] * fp[s][3];
      vm[k][4 - s] = L[k * 4 + 0] * fm[s + 1][0] + L[k * 4 + 1] * fm[s + 1][1] + L[k * 4 + 2] * fm[s + 1][2] +
                     L[k * 4 + 3] * fm[s + 1][3];
      if (fabs(vp[k][s]) > scale) scale = fabs(vp[k][s]);
      if (fabs(vm[k][4 - s]) > scale) scale = fabs(vm[k][4 - s]);
    }
  double dev = 0.0;
  for (int k = 0; k < 4; ++k) {
    const double a = face_side_deviation(vp[k], scale), b = face_side_deviation(vm[k], scale);
    if (a > dev) dev = a;
    if (b > dev) dev = b;
  }
  return dev;
}

void orc_cell_labels(const orc_grid *g, const double *U, unsigned char *labels) {
  orc_cell_labels_at(g, U, labels, 1e-2);
}

/* The same with the deviation above which a node is labelled as a
 * parameter. */
void orc_cell_labels_at(const orc_grid *g, const double *U, unsigned char *labels, double deviation) {
  for (int i = 0; i < g->nx; ++i)
    for (int j = 0; j < g->ny; ++j) {
      const int ei = ORC_NG + i, ej = ORC_NG + j;
      double dev = face_deviation(g, U, 0, ei, ej);
      double d2 = face_deviation(g, U, 0, ei + 1, ej);
      if (d2 > dev) dev = d2;
      d2 = face_deviation(g, U, 1, ei, ej);
      if (d2 > dev) dev = d2;
      d2 = face_deviation(g, U, 1, ei, ej + 1);
      if (d2 > dev) dev = d2;
      labels[(size_t)i * g->ny + j] = dev > deviation;
    }
}
