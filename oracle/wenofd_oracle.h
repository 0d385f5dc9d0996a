/*
 * wenofd_oracle.h — CPU restatement of the WENO-FD per-step hot path of
 * infinity-07/FD-WENO-EulerEquation.
 *
 * TEST INFRASTRUCTURE, NOT PRODUCT.  Only tests/, the smoke() check and the
 * CPU-baseline leg of bench.py load it, and only as the checker.  The product
 * path (libwenofd) never calls it.
 *
 * Parity is pinned: the restatement is checked bit for bit against the
 * reference's own sources compiled here with -ffp-contract=off (Makefile
 * target `ref`, fixtures in tests/golden/), and against the reference's
 * published convergence table (README.md:67-74).
 *
 * Arrays follow the reference's index order m_Uh[ei][ej].vector[r] made
 * structure-of-arrays: a full state is float64 [4][NX+8][NY+8] with ej (y)
 * fastest, 4 ghost nodes on each side (src/WENOFD.cpp:36).  An interior state
 * is [4][NX][NY].
 */
#ifndef WENOFD_ORACLE_H
#define WENOFD_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_NG 4

/* BOUNDARYTYPE (utils/equations.hpp:45-51) */
enum { ORC_PERIOD = 0, ORC_SLIP = 1, ORC_SPECIAL = 2, ORC_SYMMETRIC = 3 };
/* SCHEMETYPE (utils/equations.hpp:15-21) */
enum { ORC_WENOJS = 0, ORC_WENOZ = 1, ORC_WENOZP = 2, ORC_WENOZPI = 3 };
/* TESTCASETYPE (utils/equations.hpp:30-36) plus two seeded cases that the
 * reference has no enum for: a four-quadrant Riemann problem with seeded
 * states and a periodic shear layer with seeded noise. */
enum {
  ORC_SMOOTH = 0, ORC_RIEMANN1 = 1, ORC_RIEMANN2 = 2, ORC_RTI = 3,
  ORC_RIEMANN_SEEDED = 4, ORC_SHEAR = 5
};

typedef struct orc_case {
  int testcase;
  double xl, xr, yl, yr;
  double t_end, gamma;
  int bc_left, bc_right, bc_bottom, bc_top;
  int gravity;      /* RTI gravity source (src/WENOFD.cpp:800-821) */
  int exact;        /* an exact density exists (SMOOTH) */
  double quad[16];  /* {rho,u,v,p} for (x<c,y<c), (x<c,y>=c), (x>=c,y<c), (x>=c,y>=c) */
  double interface; /* quadrant interface c */
  unsigned long long seed;
} orc_case;

typedef struct orc_grid {
  int nx, ny;       /* ELEMNUMX / ELEMNUMY: nodes including both boundary nodes */
  int scheme;
  int bc_left, bc_right, bc_bottom, bc_top;
  int gravity;
  double dx, dy, gamma;
  double zp_lambda; /* pow(dx, 2/3) for WENO-ZP (include/Utility.hpp:531) */
  double xl, yl;
  const double *special; /* SPECIAL ghost table, see orc_special_table */
} orc_grid;

/* scalar pieces */
double orc_weno5(int scheme, double a, double b, double c, double d, double e, double zp_lambda);
void orc_wenoz_weights(double a, double b, double c, double d, double e, double w[3]);
void orc_phys_flux(int dir, double gamma, const double U[4], double F[4]);
double orc_max_eig(int dir, double gamma, const double U[4]);
void orc_flux_split(int dir, double gamma, const double U[4], double fm[4], double fp[4]);
void orc_eigen_lr(int dir, double gamma, const double U[4], double L[16], double R[16]);

/* cases and grids */
void orc_case_setup(int testcase, unsigned long long seed, orc_case *c);
void orc_grid_setup(const orc_case *c, int nx, int ny, int scheme, orc_grid *g);
double orc_node_x(const orc_grid *g, int ei);
double orc_node_y(const orc_grid *g, int ej);
void orc_u0(const orc_case *c, double x, double y, double U[4]);
void orc_initial_state(const orc_case *c, const orc_grid *g, double *U);
long orc_special_table_size(const orc_grid *g);
void orc_special_table(const orc_case *c, const orc_grid *g, double *tab);

/* the hot path */
void orc_fill_boundary(const orc_grid *g, double *U);
void orc_fill_boundary_slab(const orc_grid *g, double *U, int left_edge, int right_edge);
void orc_assemble_rhs(const orc_grid *g, double *U, double *rhs);
void orc_assemble_rhs_ghosted(const orc_grid *g, const double *U, double *rhs);
int orc_calc_dt(const orc_grid *g, const double *U, double cfl, double now, double t_end, double *dt);
void orc_rk_step(const orc_grid *g, int rk, double *U, double *Un, double *rhs, double dt);
int orc_run(const orc_grid *g, int rk, double cfl, double *U, double *Un, double *rhs, double *now,
            double t_end, long max_steps, long *steps, double *dts, long dts_cap);
void orc_error_norms(const orc_grid *g, const double *U, double t, double out[3]);

void orc_conservation_sums(const orc_grid *g, const double *U, double out[4]);

/* Learned troubled-cell indicator (no reference counterpart; these restate
 * this project's own definitions, for checking the CUDA kernels):
 *  features: per interior cell, the 5x5 windows of density and pressure,
 *    each normalised as (v - v_centre) * (1 / max|v - v_centre|) (all zero when
 *    that range is <= 1e-4 (|v_centre| + 1e-12)); 50 floats, density first,
 *    window row-major in (ei, ej).  Computed in FP32 from the FP32-rounded
 *    state.  U must have its ghosts filled.
 *  labels: 1 if, at any of the cell's four faces, for any characteristic
 *    field and side, the WENO-Z nonlinear weights differ from (0.1, 0.6, 0.3)
 *    by more than 1e-2 while that stencil's values vary by more than 1e-2
 *    of the largest characteristic magnitude at the face.  FP64. */
void orc_cell_features(const orc_grid *g, const double *U, float *features);
void orc_cell_labels(const orc_grid *g, const double *U, unsigned char *labels);
void orc_cell_labels_at(const orc_grid *g, const double *U, unsigned char *labels, double deviation);

unsigned long long orc_splitmix64(unsigned long long *state);
double orc_uniform01(unsigned long long *state);

#ifdef __cplusplus
}
#endif

#endif
