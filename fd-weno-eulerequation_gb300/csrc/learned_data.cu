// Training data of the learned troubled-cell indicator (learned.cu):
//  - k_features: 5x5 windows of density and pressure per cell, normalised
//    (FP32), the network's 50 inputs;
//  - k_labels: 1 where WENO-Z's nonlinear weights leave the linear weights
//    (FP64, the training target).
// Compiled with -fmad=false: features and labels then round exactly like the
// oracle's restatement (oracle/wenofd_oracle.c), which tests hold them to.
#include "learned_common.cuh"
#include "physics.cuh"

namespace wenofd {
namespace lrn {

// ------------------------------------------------------------- features

__global__ void k_features(Geom g, const double *U, float *feat) {
  const long long n = (long long)g.nx * g.ny;
  const float gam = float(g.gamma);
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    const int i = int(c / g.ny), j = int(c - (c / g.ny) * g.ny);
    float wr[25], wp[25];
    for (int a = 0; a < 5; ++a)
      for (int b = 0; b < 5; ++b) {
        const long long base = (long long)(kGhost + i + a - 2) * g.pitch + (kGhost + j + b - 2);
        const float r = float(U[base]), mu = float(U[g.plane + base]), mv = float(U[2 * g.plane + base]),
                    E = float(U[3 * g.plane + base]);
        wr[a * 5 + b] = r;
        wp[a * 5 + b] = pressure32(gam, r, mu, mv, E);
      }
    float o[25];
    normalise(wr, o);
    for (int k = 0; k < 25; ++k) feat[c * kIn + k] = o[k];
    normalise(wp, o);
    for (int k = 0; k < 25; ++k) feat[c * kIn + 25 + k] = o[k];
  }
}

// --------------------------------------------------------------- labels

// Row k of the left eigenvectors (utils/equations.hpp:174-236) from the
// face-average state's primitives.
template <int DIR>
__device__ __forceinline__ void left_row(int k, double u, double v, double c, double B1, double B2, double l[4]) {
  const double ic = 1.0 / c, nc = (DIR == 0 ? u : v) / c;
  if (DIR == 0) {
    if (k == 0) { l[0] = (B2 + nc) / 2; l[1] = -(B1 * u + ic) / 2; l[2] = -(B1 * v) / 2; l[3] = B1 / 2; }
    if (k == 1) { l[0] = v; l[1] = 0; l[2] = -1; l[3] = 0; }
    if (k == 2) { l[0] = 1 - B2; l[1] = B1 * u; l[2] = B1 * v; l[3] = -B1; }
    if (k == 3) { l[0] = (B2 - nc) / 2; l[1] = -(B1 * u - ic) / 2; l[2] = -B1 * v / 2; l[3] = B1 / 2; }
  } else {
    if (k == 0) { l[0] = (B2 + nc) / 2; l[1] = -(B1 * u) / 2; l[2] = -(B1 * v + ic) / 2; l[3] = B1 / 2; }
    if (k == 1) { l[0] = -u; l[1] = 1; l[2] = 0; l[3] = 0; }
    if (k == 2) { l[0] = 1 - B2; l[1] = B1 * u; l[2] = B1 * v; l[3] = -B1; }
    if (k == 3) { l[0] = (B2 - nc) / 2; l[1] = -(B1 * u) / 2; l[2] = -(B1 * v - ic) / 2; l[3] = B1 / 2; }
  }
}

__device__ double side_deviation(const double v[5], double scale) {
  double lo = v[0], hi = v[0];
  for (int s = 1; s < 5; ++s) {
    lo = v[s] < lo ? v[s] : lo;
    hi = v[s] > hi ? v[s] : hi;
  }
  if (hi - lo <= 1e-2 * scale) return 0.0;
  double w0, w1, w2;
  dev::wenoz_weights<double>(v[0], v[1], v[2], v[3], v[4], w0, w1, w2);
  return fmax(fabs(w0 - 0.1), fmax(fabs(w1 - 0.6), fabs(w2 - 0.3)));
}

// Largest WENO-Z weight deviation over the characteristic fields and sides
// of the face between (ei-1, ej) and (ei, ej) (DIR 0) or (ei, ej-1), (ei, ej).
template <int DIR>
__device__ double face_deviation(const Geom &g, const double *U, int ei, int ej) {
  const int di = DIR == 0 ? 1 : 0, dj = DIR == 0 ? 0 : 1;
  double ave[4];
  for (int r = 0; r < 4; ++r)
    ave[r] = 0.5 * (U[r * g.plane + (long long)(ei - di) * g.pitch + (ej - dj)] +
                    U[r * g.plane + (long long)ei * g.pitch + ej]);
  double u, v, p;
  dev::primitives<double>(g.gamma, ave, u, v, p);
  const double c = sqrt(g.gamma * p / ave[0]);
  const double B1 = (g.gamma - 1) / (c * c);
  const double B2 = B1 * (u * u + v * v) / 2;
  double fp[6][4], fm[6][4];
  for (int s = 0; s < 6; ++s) {
    double q[4];
    for (int r = 0; r < 4; ++r) q[r] = U[r * g.plane + (long long)(ei + (s - 3) * di) * g.pitch + (ej + (s - 3) * dj)];
    dev::flux_split<double, DIR>(g.gamma, q, fm[s], fp[s]);
  }
  double vp[4][5], vm[4][5], scale = 0.0;
  for (int k = 0; k < 4; ++k) {
    double l[4];
    left_row<DIR>(k, u, v, c, B1, B2, l);
    for (int s = 0; s < 5; ++s) {
      vp[k][s] = l[0] * fp[s][0] + l[1] * fp[s][1] + l[2] * fp[s][2] + l[3] * fp[s][3];
      vm[k][4 - s] = l[0] * fm[s + 1][0] + l[1] * fm[s + 1][1] + l[2] * fm[s + 1][2] + l[3] * fm[s + 1][3];
      scale = fmax(scale, fmax(fabs(vp[k][s]), fabs(vm[k][4 - s])));
    }
  }
  double dev = 0.0;
  for (int k = 0; k < 4; ++k) dev = fmax(dev, fmax(side_deviation(vp[k], scale), side_deviation(vm[k], scale)));
  return dev;
}

__global__ void k_labels(Geom g, const double *U, unsigned char *labels, double deviation) {
  const long long n = (long long)g.nx * g.ny;
  for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += (long long)gridDim.x * blockDim.x) {
    const int ei = kGhost + int(c / g.ny), ej = kGhost + int(c - (c / g.ny) * g.ny);
    double d = face_deviation<0>(g, U, ei, ej);
    d = fmax(d, face_deviation<0>(g, U, ei + 1, ej));
    d = fmax(d, face_deviation<1>(g, U, ei, ej));
    d = fmax(d, face_deviation<1>(g, U, ei, ej + 1));
    labels[c] = d > deviation ? 1 : 0;
  }
}


}  // namespace lrn

cudaError_t launch_features(const Geom &g, const double *U, float *feat, cudaStream_t s) {
  lrn::k_features<<<lrn::grid_for((long long)g.nx * g.ny, 128, 152 * 32), 128, 0, s>>>(g, U, feat);
  return cudaGetLastError();
}

cudaError_t launch_labels(const Geom &g, const double *U, unsigned char *labels, double deviation, cudaStream_t s) {
  lrn::k_labels<<<lrn::grid_for((long long)g.nx * g.ny, 128, 152 * 32), 128, 0, s>>>(g, U, labels, deviation);
  return cudaGetLastError();
}

}  // namespace wenofd
