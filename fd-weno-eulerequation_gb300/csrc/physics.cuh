// Device physics of the WENO-FD hot path, templated on the arithmetic type.
//
// With T = double and the translation unit built with -fmad=false, every
// expression below rounds exactly like the reference compiled without FMA
// contraction: operands are combined in the reference's evaluation order
// (C++ left-to-right), divisions and square roots are IEEE correctly rounded,
// and common subexpressions are shared only where the reference computes the
// identical operation on identical operands.  Citations are to files of
// infinity-07/FD-WENO-EulerEquation.
#pragma once

#include "wenofd_internal.h"

namespace wenofd {
namespace dev {

__device__ __forceinline__ double tsqrt(double x) { return sqrt(x); }
// FP32: the units of the FP32 forms are compiled with -prec-sqrt=false, so
// this is the hardware approximation there (about 1 ulp).
__device__ __forceinline__ float tsqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double tabs(double x) { return fabs(x); }
__device__ __forceinline__ float tabs(float x) { return fabsf(x); }

// Division.  FP64: IEEE '/'.  FP32 form: __fdividef, reciprocal times
// numerator (about 2 ulp; the FP32 form is not bitwise and does not need
// IEEE rounding).
__device__ __forceinline__ double tdiv(double a, double b) { return a / b; }
__device__ __forceinline__ float tdiv(float a, float b) { return __fdividef(a, b); }

// Pressure from conserved variables (utils/equations.hpp:108-112):
// p = (gamma - 1) * (E - 0.5 * rho * (u*u + v*v)), u = U1/U0, v = U2/U0.
template <typename T>
__device__ __forceinline__ void primitives(T gamma, const T U[4], T &u, T &v, T &p) {
  u = tdiv(U[1], U[0]);
  v = tdiv(U[2], U[0]);
  p = (gamma - T(1.0)) * (U[3] - T(0.5) * U[0] * (u * u + v * v));
}

// fluxSplitX / fluxSplitY (utils/equations.hpp:365-393) with getPhyFluxX/Y
// (105-134) and getMaxEigenValueX/Y (149-171): pointwise Lax-Friedrichs,
// F+- = 0.5 * (F +- (|u_n| + c) U).
template <typename T, int DIR>
__device__ __forceinline__ void flux_split(T gamma, const T U[4], T fm[4], T fp[4]) {
  T u, v, p;
  primitives(gamma, U, u, v, p);
  const T rho = U[0], E = U[3];
  T F[4];
  if (DIR == 0) {
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
  const T c = tsqrt(tdiv(gamma * p, rho));
  const T ws = (DIR == 0 ? tabs(u) : tabs(v)) + c;
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    fm[r] = T(0.5) * (F[r] - ws * U[r]);
    fp[r] = T(0.5) * (F[r] + ws * U[r]);
  }
}

// Packed FP32 pairs: Blackwell issues two FP32 adds, multiplies or FMAs of a
// float2 as one instruction (round-to-nearest each, as the scalar forms).
// The FP32 forms run independent chains on pairs: the (x, y) and (z, w)
// halves of a node's float4 (stage_f32.cuh), and the two sides of a
// characteristic field's reconstruction (weno2 below).
__device__ __forceinline__ float2 lo2(const float4 v) { return make_float2(v.x, v.y); }
__device__ __forceinline__ float2 hi2(const float4 v) { return make_float2(v.z, v.w); }
__device__ __forceinline__ float4 join2(const float2 a, const float2 b) { return make_float4(a.x, a.y, b.x, b.y); }
__device__ __forceinline__ float2 splat2(float a) { return make_float2(a, a); }
// a - b, exactly as the scalar subtraction rounds it
__device__ __forceinline__ float2 sub2(const float2 a, const float2 b) { return __ffma2_rn(b, splat2(-1.0f), a); }

// ---------------------------------------------------------------- WENO

// Smoothness indicators shared by all four schemes (include/Utility.hpp
// 427-437, 465-475): beta = 13/12 t1^2 + 1/4 t2^2 evaluated as
// ((13/12*t1)*t1) + ((1/4*t2)*t2).
template <typename T>
__device__ __forceinline__ void betas(T a, T b, T c, T d, T e, T &bm, T &b0, T &bp) {
  const T c1312 = T(13.0 / 12.0), c14 = T(0.25);
  T t1 = (a - T(2.0) * b + c);
  T t2 = (a - T(4.0) * b + T(3.0) * c);
  bm = c1312 * t1 * t1 + c14 * t2 * t2;
  t1 = (b - T(2.0) * c + d);
  t2 = (b - d);
  b0 = c1312 * t1 * t1 + c14 * t2 * t2;
  t1 = (c - T(2.0) * d + e);
  t2 = (T(3.0) * c - T(4.0) * d + e);
  bp = c1312 * t1 * t1 + c14 * t2 * t2;
}

// Candidate values p0..p2 at x_{i+1/2} (include/Utility.hpp:499-501).
template <typename T>
__device__ __forceinline__ T combine(T w0, T w1, T w2, T a, T b, T c, T d, T e) {
  const T c13 = T(1.0 / 3.0), c16 = T(1.0 / 6.0), c56 = T(5.0 / 6.0), c76 = T(7.0 / 6.0), c116 = T(11.0 / 6.0);
  const T p0 = c13 * a - c76 * b + c116 * c;
  const T p1 = -c16 * b + c56 * c + c13 * d;
  const T p2 = c13 * c + c56 * d - c16 * e;
  return w0 * p0 + w1 * p1 + w2 * p2;
}

// WENO-JS, include/Utility.hpp:415-456 (eps = 1e-6).
template <typename T>
__device__ __forceinline__ T weno_js(T a, T b, T c, T d, T e) {
  T b0, b1, b2;
  betas(a, b, c, d, e, b0, b1, b2);
  const T eps = T(1.0e-6);
  T w0 = tdiv(T(0.1), ((eps + b0) * (eps + b0)));
  T w1 = tdiv(T(0.6), ((eps + b1) * (eps + b1)));
  T w2 = tdiv(T(0.3), ((eps + b2) * (eps + b2)));
  const T sum = w0 + w1 + w2;
  w0 = tdiv(w0, sum);
  w1 = tdiv(w1, sum);
  w2 = tdiv(w2, sum);
  return combine(w0, w1, w2, a, b, c, d, e);
}

// WENO-Z, include/Utility.hpp:457-504 (eps = 1e-20).
//
// FP64: the weight products are taken left to right, tau*inv*tau*inv, as in
// the reference (lines 489-491), with no guard.  FP32: (tau/(beta+1e-20))^2
// overflows where a stencil is exactly flat (beta = 0) next to a jump, so the
// ratio r is capped at 1e18 before squaring (r^2 <= 1e36 stays finite); a
// weight that large already makes its stencil's normalised weight 1 to FP32
// precision, so the cap changes nothing else.
template <typename T>
__device__ __forceinline__ void wenoz_weights(T a, T b, T c, T d, T e, T &w0, T &w1, T &w2) {
  T bm, b0, bp;
  betas(a, b, c, d, e, bm, b0, bp);
  const T eps = T(1.0e-20);
  const T ibm = tdiv(T(1.0), (bm + eps));
  const T ib0 = tdiv(T(1.0), (b0 + eps));
  const T ibp = tdiv(T(1.0), (bp + eps));
  const T tau = tabs(bm - bp);
  if constexpr (sizeof(T) == 4) {
    const T rm = fminf(tau * ibm, 1.0e18f), r0 = fminf(tau * ib0, 1.0e18f), rp = fminf(tau * ibp, 1.0e18f);
    w0 = T(0.1) * (T(1.0) + rm * rm);
    w1 = T(0.6) * (T(1.0) + r0 * r0);
    w2 = T(0.3) * (T(1.0) + rp * rp);
  } else {
    w0 = T(0.1) * (T(1.0) + (tau * ibm * tau * ibm));
    w1 = T(0.6) * (T(1.0) + (tau * ib0 * tau * ib0));
    w2 = T(0.3) * (T(1.0) + (tau * ibp * tau * ibp));
  }
  const T ws = w0 + w1 + w2;
  w0 = tdiv(w0, ws);
  w1 = tdiv(w1, ws);
  w2 = tdiv(w2, ws);
}

template <typename T>
__device__ __forceinline__ T weno_z(T a, T b, T c, T d, T e) {
  T w0, w1, w2;
  wenoz_weights(a, b, c, d, e, w0, w1, w2);
  return combine(w0, w1, w2, a, b, c, d, e);
}

// pow(x, 2) of the reference's ZP/ZPI weights is evaluated as x*x, the
// correctly rounded square.  glibc's pow(x, 2) differs from it by one ulp on
// about 0.1% of inputs, so WENO-ZP/ZPI agree with the reference to rounding
// rather than bit for bit (WENO-JS and WENO-Z have no pow).
template <typename T> __device__ __forceinline__ T sq(T x) { return x * x; }

// FP32 ZP/ZPI: eps = 1e-40 is subnormal in FP32 and the weight ratios can
// exceed the FP32 range, so the FP32 form divides with IEEE '/' (subnormal
// safe) and caps each ratio term at 1e18 before it is squared or summed.
template <typename T> __device__ __forceinline__ T zdiv(T a, T b) { return tdiv(a, b); }
template <> __device__ __forceinline__ float zdiv<float>(float a, float b) { return fminf(a / b, 1.0e18f); }

// WENO-ZP, include/Utility.hpp:505-558 (eps = 1e-40; lambda = pow(dx, 2/3)).
template <typename T>
__device__ __forceinline__ T weno_zp(T a, T b, T c, T d, T e, T lambda) {
  T bm, b0, bp;
  betas(a, b, c, d, e, bm, b0, bp);
  const T tau = tabs(bm - bp);
  const T eps = T(1.0e-40);
  T w0 = T(0.1) * (T(1) + sq(zdiv((tau + eps), (bm + eps))) + zdiv(lambda * (bm + eps), (tau + eps)));
  T w1 = T(0.6) * (T(1) + sq(zdiv((tau + eps), (b0 + eps))) + zdiv(lambda * (b0 + eps), (tau + eps)));
  T w2 = T(0.3) * (T(1) + sq(zdiv((tau + eps), (bp + eps))) + zdiv(lambda * (bp + eps), (tau + eps)));
  const T sum = w0 + w1 + w2;
  w0 = tdiv(w0, sum);
  w1 = tdiv(w1, sum);
  w2 = tdiv(w2, sum);
  return combine(w0, w1, w2, a, b, c, d, e);
}

// WENO-ZPI, include/Utility.hpp:559-615 (lambda = 3.3, eps = 1e-40).
template <typename T>
__device__ __forceinline__ T weno_zpi(T a, T b, T c, T d, T e) {
  T bm, b0, bp;
  betas(a, b, c, d, e, bm, b0, bp);
  const T tau = tabs(bm - bp);
  const T lambda = T(3.3);
  const T mx_in = (b0 < bp) ? bp : b0;  // std::max(beta, betap)
  const T bmax = (bm < mx_in) ? mx_in : bm;
  const T mn_in = (bp < b0) ? bp : b0;  // std::min(beta, betap)
  const T bmin = (mn_in < bm) ? mn_in : bm;
  const T alpha = T(1) - zdiv(bmin, (bmax + T(1e-40)));
  const T eps = T(1.0e-40);
  T w0 = T(0.1) * (T(1) + sq(zdiv(tau, (bm + eps))) + zdiv(lambda * alpha * (bm), (bmax + eps)));
  T w1 = T(0.6) * (T(1) + sq(zdiv(tau, (b0 + eps))) + zdiv(lambda * alpha * (b0), (bmax + eps)));
  T w2 = T(0.3) * (T(1) + sq(zdiv(tau, (bp + eps))) + zdiv(lambda * alpha * (bp), (bmax + eps)));
  const T sum = w0 + w1 + w2;
  w0 = tdiv(w0, sum);
  w1 = tdiv(w1, sum);
  w2 = tdiv(w2, sum);
  return combine(w0, w1, w2, a, b, c, d, e);
}

// CWENOFD::useWENO (src/WENOFD.cpp:823-848), scheme fixed at compile time.
template <typename T, int SCHEME>
__device__ __forceinline__ T weno(T a, T b, T c, T d, T e, T zp_lambda) {
  if (SCHEME == kWenoJS) return weno_js(a, b, c, d, e);
  if (SCHEME == kWenoZ) return weno_z(a, b, c, d, e);
  if (SCHEME == kWenoZP) return weno_zp(a, b, c, d, e, zp_lambda);
  return weno_zpi(a, b, c, d, e);
}

// WENO-JS / WENO-Z on two stencils at once (betas, wenoz_weights or the
// WENO-JS weights, and combine of physics.cuh, in the same order), used for
// the + and - sides of one characteristic field: the arithmetic runs on packed
// pairs, the reciprocals and the caps per element.
__device__ __forceinline__ void betas2(float2 a, float2 b, float2 c, float2 d, float2 e, float2 &bm, float2 &b0,
                                       float2 &bp) {
  const float2 c1312 = splat2(float(13.0 / 12.0)), c14 = splat2(0.25f), m2 = splat2(-2.0f), m4 = splat2(-4.0f),
               p3 = splat2(3.0f);
  float2 t1 = __fadd2_rn(__ffma2_rn(m2, b, a), c);
  float2 t2 = __ffma2_rn(p3, c, __ffma2_rn(m4, b, a));
  bm = __ffma2_rn(__fmul2_rn(c1312, t1), t1, __fmul2_rn(__fmul2_rn(c14, t2), t2));
  t1 = __fadd2_rn(__ffma2_rn(m2, c, b), d);
  t2 = sub2(b, d);
  b0 = __ffma2_rn(__fmul2_rn(c1312, t1), t1, __fmul2_rn(__fmul2_rn(c14, t2), t2));
  t1 = __fadd2_rn(__ffma2_rn(m2, d, c), e);
  t2 = __fadd2_rn(__ffma2_rn(m4, d, __fmul2_rn(p3, c)), e);
  bp = __ffma2_rn(__fmul2_rn(c1312, t1), t1, __fmul2_rn(__fmul2_rn(c14, t2), t2));
}

__device__ __forceinline__ float2 rcp2(float2 x) { return make_float2(__fdividef(1.0f, x.x), __fdividef(1.0f, x.y)); }

template <int SCHEME>
__device__ __forceinline__ float2 weno2(float2 a, float2 b, float2 c, float2 d, float2 e) {
  static_assert(SCHEME == kWenoJS || SCHEME == kWenoZ, "packed WENO-JS and WENO-Z only");
  float2 bm, b0, bp, w0, w1, w2;
  betas2(a, b, c, d, e, bm, b0, bp);
  if constexpr (SCHEME == kWenoZ) {
    const float2 eps = splat2(1.0e-20f), one = splat2(1.0f);
    const float2 ibm = rcp2(__fadd2_rn(bm, eps)), ib0 = rcp2(__fadd2_rn(b0, eps)), ibp = rcp2(__fadd2_rn(bp, eps));
    const float2 tau = make_float2(fabsf(bm.x - bp.x), fabsf(bm.y - bp.y));
    float2 rm = __fmul2_rn(tau, ibm), r0 = __fmul2_rn(tau, ib0), rp = __fmul2_rn(tau, ibp);
    rm = make_float2(fminf(rm.x, 1.0e18f), fminf(rm.y, 1.0e18f));
    r0 = make_float2(fminf(r0.x, 1.0e18f), fminf(r0.y, 1.0e18f));
    rp = make_float2(fminf(rp.x, 1.0e18f), fminf(rp.y, 1.0e18f));
    w0 = __fmul2_rn(splat2(0.1f), __ffma2_rn(rm, rm, one));
    w1 = __fmul2_rn(splat2(0.6f), __ffma2_rn(r0, r0, one));
    w2 = __fmul2_rn(splat2(0.3f), __ffma2_rn(rp, rp, one));
  } else {
    const float2 eps = splat2(1.0e-6f);
    const float2 sm = __fadd2_rn(eps, bm), s0 = __fadd2_rn(eps, b0), sp = __fadd2_rn(eps, bp);
    w0 = __fmul2_rn(splat2(0.1f), rcp2(__fmul2_rn(sm, sm)));
    w1 = __fmul2_rn(splat2(0.6f), rcp2(__fmul2_rn(s0, s0)));
    w2 = __fmul2_rn(splat2(0.3f), rcp2(__fmul2_rn(sp, sp)));
  }
  const float2 iws = rcp2(__fadd2_rn(__fadd2_rn(w0, w1), w2));
  w0 = __fmul2_rn(w0, iws);
  w1 = __fmul2_rn(w1, iws);
  w2 = __fmul2_rn(w2, iws);
  const float2 c13 = splat2(float(1.0 / 3.0)), c56 = splat2(float(5.0 / 6.0)), c116 = splat2(float(11.0 / 6.0));
  const float2 mc76 = splat2(-float(7.0 / 6.0)), mc16 = splat2(-float(1.0 / 6.0));
  const float2 q0 = __ffma2_rn(c116, c, __ffma2_rn(mc76, b, __fmul2_rn(c13, a)));
  const float2 q1 = __ffma2_rn(c13, d, __ffma2_rn(c56, c, __fmul2_rn(mc16, b)));
  const float2 q2 = __ffma2_rn(mc16, e, __ffma2_rn(c56, d, __fmul2_rn(c13, c)));
  return __ffma2_rn(w2, q2, __ffma2_rn(w1, q1, __fmul2_rn(w0, q0)));
}

// The two sides of one characteristic field at a face: the + side on F+
// stencil values p0..p4, the - side on F- values mirrored (m4..m0), summed.
// FP64 evaluates them one after the other as the reference does; FP32
// WENO-JS and WENO-Z evaluate both at once on packed pairs.
template <typename T, int SCHEME>
__device__ __forceinline__ T weno_sides(const T vp[5], const T vm[5], T zp_lambda) {
  if constexpr (sizeof(T) == 4 && (SCHEME == kWenoJS || SCHEME == kWenoZ)) {
    const float2 r = weno2<SCHEME>(make_float2(vp[0], vm[4]), make_float2(vp[1], vm[3]), make_float2(vp[2], vm[2]),
                                   make_float2(vp[3], vm[1]), make_float2(vp[4], vm[0]));
    return r.x + r.y;
  } else {
    const T hp = weno<T, SCHEME>(vp[0], vp[1], vp[2], vp[3], vp[4], zp_lambda);
    const T hm = weno<T, SCHEME>(vm[4], vm[3], vm[2], vm[1], vm[0], zp_lambda);
    return hp + hm;
  }
}

// ------------------------------------------------------- one face flux

// Characteristic WENO flux at one face (src/WENOFD.cpp:526-643 in x,
// 668-791 in y): average state of the two nodes, L and R of the x- or
// y-Jacobian there (utils/equations.hpp:174-299), five projected F+ (nodes
// face-3..face+1) and five F- (face-2..face+2), one WENO per characteristic
// field and side (minus side mirrored), back-projection.  L and R are built
// from one set of (u, v, p, c, B1, B2, H): the reference recomputes them per
// matrix from the same inputs, which gives identical values.
//
// fp(s, r) / fm(s, r): component r of F+ at node face-3+s and of F- at node
// face-2+s, s = 0..4.
template <typename T>
struct StridedStencil {  // SoA: nodes `ss` elements apart, components `cs` apart
  const T *p;
  int ss, cs;
  __device__ __forceinline__ T operator()(int s, int r) const { return p[s * ss + r * cs]; }
};
struct Float4Stencil {  // AoS: one float4 per node, nodes `ss` float4s apart
  const float4 *p;
  int ss;
  __device__ __forceinline__ float operator()(int s, int r) const {
    const float4 v = p[s * ss];
    return r == 0 ? v.x : (r == 1 ? v.y : (r == 2 ? v.z : v.w));
  }
};

template <typename T, int DIR, int SCHEME, typename St>
__device__ __forceinline__ void face_flux_st(T gamma, T zp_lambda, const T um[4], const T u0[4], const St &fp,
                                             const St &fm, T out[4]);

// fp / fm point at F+ of node face-3 and F- of node face-2, component 0;
// consecutive stencil nodes are `ss` elements apart, components `cs` apart.
template <typename T, int DIR, int SCHEME>
__device__ __forceinline__ void face_flux(T gamma, T zp_lambda, const T um[4], const T u0[4],
                                          const T *fp, const T *fm, int ss, int cs, T out[4]) {
  face_flux_st<T, DIR, SCHEME>(gamma, zp_lambda, um, u0, StridedStencil<T>{fp, ss, cs},
                               StridedStencil<T>{fm, ss, cs}, out);
}

template <typename T, int DIR, int SCHEME, typename St>
__device__ __forceinline__ void face_flux_st(T gamma, T zp_lambda, const T um[4], const T u0[4], const St &fp,
                                             const St &fm, T out[4]) {
  T ave[4];
#pragma unroll
  for (int r = 0; r < 4; ++r) ave[r] = T(0.5) * (um[r] + u0[r]);
  T u, v, p;
  primitives(gamma, ave, u, v, p);
  const T rho = ave[0], E = ave[3];
  const T c = tsqrt(tdiv(gamma * p, rho));
  const T B1 = tdiv((gamma - T(1)), (c * c));
  const T B2 = B1 * (u * u + v * v) * T(0.5);
  const T H = tdiv((E + p), rho);
  const T ic = tdiv(T(1.0), c);
  const T nc = tdiv(DIR == 0 ? u : v, c);  // u/c in x, v/c in y
  const T B1u = B1 * u, B1v = B1 * v;

  T vh[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    T l0, l1, l2, l3;  // row k of the left eigenvector matrix
    if (DIR == 0) {
      if (k == 0) { l0 = (B2 + nc) * T(0.5); l1 = -(B1u + ic) * T(0.5); l2 = -(B1v) * T(0.5); l3 = B1 * T(0.5); }
      if (k == 1) { l0 = v; l1 = T(0); l2 = T(-1); l3 = T(0); }
      if (k == 2) { l0 = (T(1) - B2); l1 = B1u; l2 = B1v; l3 = -B1; }
      if (k == 3) { l0 = (B2 - nc) * T(0.5); l1 = -(B1u - ic) * T(0.5); l2 = -B1v * T(0.5); l3 = B1 * T(0.5); }
    } else {
      if (k == 0) { l0 = (B2 + nc) * T(0.5); l1 = -(B1u) * T(0.5); l2 = -(B1v + ic) * T(0.5); l3 = B1 * T(0.5); }
      if (k == 1) { l0 = -u; l1 = T(1); l2 = T(0); l3 = T(0); }
      if (k == 2) { l0 = T(1) - B2; l1 = B1u; l2 = B1v; l3 = -B1; }
      if (k == 3) { l0 = (B2 - nc) * T(0.5); l1 = -(B1u) * T(0.5); l2 = -(B1v - ic) * T(0.5); l3 = B1 * T(0.5); }
    }
    T vp[5], vm[5];
#pragma unroll
    for (int s = 0; s < 5; ++s) {
      T x = l0 * fp(s, 0);
      x += l1 * fp(s, 1);
      x += l2 * fp(s, 2);
      x += l3 * fp(s, 3);
      vp[s] = x;
      T y = l0 * fm(s, 0);
      y += l1 * fm(s, 1);
      y += l2 * fm(s, 2);
      y += l3 * fm(s, 3);
      vm[s] = y;
    }
    vh[k] = weno_sides<T, SCHEME>(vp, vm, zp_lambda);
  }

  // R * vh, rows in the reference's order (utils/equations.hpp:239-299).
  const T q2 = (u * u + v * v) * T(0.5);
  T R[4][4];
  if (DIR == 0) {
    R[0][0] = T(1);      R[0][1] = T(0);  R[0][2] = T(1); R[0][3] = T(1);
    R[1][0] = u - c;     R[1][1] = T(0);  R[1][2] = u;    R[1][3] = u + c;
    R[2][0] = v;         R[2][1] = T(-1); R[2][2] = v;    R[2][3] = v;
    R[3][0] = H - c * u; R[3][1] = -v;    R[3][2] = q2;   R[3][3] = H + c * u;
  } else {
    R[0][0] = T(1);      R[0][1] = T(0);  R[0][2] = T(1); R[0][3] = T(1);
    R[1][0] = u;         R[1][1] = T(1);  R[1][2] = u;    R[1][3] = u;
    R[2][0] = v - c;     R[2][1] = T(0);  R[2][2] = v;    R[2][3] = v + c;
    R[3][0] = H - c * v; R[3][1] = u;     R[3][2] = q2;   R[3][3] = H + c * v;
  }
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    T f = R[r][0] * vh[0];
    f += R[r][1] * vh[1];
    f += R[r][2] * vh[2];
    f += R[r][3] * vh[3];
    out[r] = f;
  }
}

}  // namespace dev
}  // namespace wenofd
