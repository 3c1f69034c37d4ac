// Perfect-gas thermodynamics and the three face fluxes of BES, written once as templates on
// the scalar type T (double for the residual, float for the FP32 Jacobian of the defect
// correction, Dual<N> for forward-mode Jacobians — the device counterpart of the
// reference's Eigen::AutoDiffScalar instantiation, src/FluxJacobianWrapper.tpp:32-82).
//
// The algebra is the reference's (src/FluxRoe.tpp, src/FluxFreestream.tpp,
// src/FluxSlipWall.tpp, src/GasPerfect.tpp) with its redundant work removed: each density is
// inverted once, the square roots of the two densities are taken once, the per-side sound
// speed and q^2 that the Roe flux never uses are skipped, and the wave strengths share one
// reciprocal of c^2.  Results agree with the reference to rounding (a few ulp).
#pragma once
#include <cmath>

#ifdef __CUDACC__
#define BES_HD __host__ __device__ __forceinline__
#else
#define BES_HD inline
#endif

namespace bes {

// Gas constants derived exactly as GasPerfect_::initialize (src/GasPerfect.tpp:22-28).
struct GasConst {
  double gamma, R, cv, cp, gm1;
  double inv_cv;
  double gamma_R;  // gamma * R: the true sound speed is sqrt(gamma R T)
  double harten;
};

inline GasConst make_gas(double R, double gamma, double harten) {
  GasConst g;
  g.R = R;
  g.gamma = gamma;
  g.cv = R / (gamma - 1.0);
  g.cp = g.cv + R;
  g.gm1 = gamma - 1.0;
  g.inv_cv = 1.0 / g.cv;
  g.gamma_R = gamma * R;
  g.harten = harten;
  return g;
}

// ------------------------------------------------------------------------------------
// forward-mode dual number with N derivative slots
// ------------------------------------------------------------------------------------
template <int N, class S = double>
struct Dual {
  S v;
  S d[N];
  BES_HD Dual() : v(0) {
#pragma unroll
    for (int i = 0; i < N; ++i) d[i] = 0;
  }
  BES_HD Dual(S x) : v(x) {  // NOLINT
#pragma unroll
    for (int i = 0; i < N; ++i) d[i] = 0;
  }
};
#define BES_DUAL template <int N, class S>
BES_DUAL BES_HD Dual<N, S> operator+(const Dual<N, S>& a, const Dual<N, S>& b) {
  Dual<N, S> r(a.v + b.v);
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] + b.d[i];
  return r;
}
BES_DUAL BES_HD Dual<N, S> operator-(const Dual<N, S>& a, const Dual<N, S>& b) {
  Dual<N, S> r(a.v - b.v);
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - b.d[i];
  return r;
}
BES_DUAL BES_HD Dual<N, S> operator-(const Dual<N, S>& a) {
  Dual<N, S> r(-a.v);
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = -a.d[i];
  return r;
}
BES_DUAL BES_HD Dual<N, S> operator*(const Dual<N, S>& a, const Dual<N, S>& b) {
  Dual<N, S> r(a.v * b.v);
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
  return r;
}
BES_DUAL BES_HD Dual<N, S> operator*(const Dual<N, S>& a, S b) {
  Dual<N, S> r(a.v * b);
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b;
  return r;
}
BES_DUAL BES_HD Dual<N, S> operator*(S a, const Dual<N, S>& b) { return b * a; }
BES_DUAL BES_HD Dual<N, S> operator+(const Dual<N, S>& a, S b) {
  Dual<N, S> r(a);
  r.v = a.v + b;
  return r;
}
BES_DUAL BES_HD Dual<N, S> operator+(S a, const Dual<N, S>& b) { return b + a; }
BES_DUAL BES_HD Dual<N, S> operator-(const Dual<N, S>& a, S b) {
  Dual<N, S> r(a);
  r.v = a.v - b;
  return r;
}
BES_DUAL BES_HD Dual<N, S> operator-(S a, const Dual<N, S>& b) {
  Dual<N, S> r(a - b.v);
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = -b.d[i];
  return r;
}
BES_DUAL BES_HD Dual<N, S> recip(const Dual<N, S>& a) {  // 1/a
  Dual<N, S> r(S(1) / a.v);
  const S k = -r.v * r.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * k;
  return r;
}
BES_DUAL BES_HD Dual<N, S> operator/(const Dual<N, S>& a, const Dual<N, S>& b) {
  return a * recip(b);
}
BES_DUAL BES_HD Dual<N, S> bsqrt(const Dual<N, S>& a) {
  Dual<N, S> r(std::sqrt(a.v));
  const S h = S(0.5) / r.v;
#pragma unroll
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * h;
  return r;
}
BES_DUAL BES_HD Dual<N, S> babs(const Dual<N, S>& a) {
  Dual<N, S> r(a);
  if (a.v < 0) r = -a;
  return r;
}
BES_DUAL BES_HD bool operator>(const Dual<N, S>& a, const Dual<N, S>& b) { return a.v > b.v; }
BES_DUAL BES_HD bool operator<=(const Dual<N, S>& a, const Dual<N, S>& b) { return a.v <= b.v; }
BES_DUAL BES_HD bool operator>=(const Dual<N, S>& a, const Dual<N, S>& b) { return a.v >= b.v; }
BES_DUAL BES_HD bool operator>=(const Dual<N, S>& a, S b) { return a.v >= b; }
BES_DUAL BES_HD bool operator<(const Dual<N, S>& a, S b) { return a.v < b; }
BES_DUAL BES_HD bool operator<=(const Dual<N, S>& a, S b) { return a.v <= b; }
BES_DUAL BES_HD bool operator>(const Dual<N, S>& a, S b) { return a.v > b; }

template <class T> struct ScalarOf { typedef T type; };
template <int N, class S> struct ScalarOf<Dual<N, S> > { typedef S type; };

BES_HD double recip(double a) { return 1.0 / a; }
BES_HD float recip(float a) { return 1.0f / a; }
BES_HD double babs(double a) { return std::fabs(a); }
BES_HD float babs(float a) { return std::fabs(a); }
BES_HD double bsqrt(double a) { return std::sqrt(a); }
BES_HD float bsqrt(float a) { return std::sqrt(a); }

// ------------------------------------------------------------------------------------
// per-side state used by all fluxes
// ------------------------------------------------------------------------------------
template <class T>
struct Side {
  T rho, ir;    // density, 1/density
  T u[3];       // velocity
  T e;          // internal energy per volume: rhoE - |rho u|^2 / (2 rho)
  T p;          // pressure (gamma-1) e            (GasPerfect.tpp:48-64)
  T H;          // total enthalpy (rhoE + p)/rho   (GasPerfect.tpp:141-146)
  T vn;         // normal velocity
};

template <class T>
BES_HD void make_side(const GasConst& g, const T* U, const double* n, Side<T>& s) {
  typedef typename ScalarOf<T>::type S;
  s.rho = U[0];
  s.ir = recip(U[0]);
  s.u[0] = U[1] * s.ir;
  s.u[1] = U[2] * s.ir;
  s.u[2] = U[3] * s.ir;
  const T k = U[1] * U[1] + U[2] * U[2] + U[3] * U[3];
  s.e = U[4] - k * (S(0.5) * s.ir);
  s.p = S(g.gm1) * s.e;
  s.H = (U[4] + s.p) * s.ir;
  s.vn = s.u[0] * S(n[0]) + s.u[1] * S(n[1]) + s.u[2] * S(n[2]);
}

// Euler flux from conserved variables and pressure (GasPerfect_::computeAllFlux, :266-291;
// the energy flux rho (cp T + q^2/2) vn equals (rhoE + p) vn).
template <class T>
BES_HD void euler_flux(const T* U, const Side<T>& s, const double* n, T* F) {
  typedef typename ScalarOf<T>::type S;
  F[0] = U[0] * s.vn;
  F[1] = U[1] * s.vn + s.p * S(n[0]);
  F[2] = U[2] * s.vn + s.p * S(n[1]);
  F[3] = U[3] * s.vn + s.p * S(n[2]);
  F[4] = (U[4] + s.p) * s.vn;
}

// Roe flux-difference splitting with Harten's entropy fix (FluxRoe_::computeFlux,
// src/FluxRoe.tpp:307-333).  F is per unit area.
template <class T>
BES_HD void roe_flux(const GasConst& g, const T* UL, const T* UR, const double* n, T* F) {
  typedef typename ScalarOf<T>::type S;
  Side<T> L, R;
  make_side(g, UL, n, L);
  make_side(g, UR, n, R);
  // Roe averages (FluxRoe.tpp:110-143)
  const T sL = bsqrt(L.rho), sR = bsqrt(R.rho);
  const T iden = recip(sL + sR);
  const T rho = sL * sR;
  T ua[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) ua[d] = (L.u[d] * sL + R.u[d] * sR) * iden;
  const T H = (L.H * sL + R.H * sR) * iden;
  const T q2 = ua[0] * ua[0] + ua[1] * ua[1] + ua[2] * ua[2];
  const T vn = ua[0] * S(n[0]) + ua[1] * S(n[1]) + ua[2] * S(n[2]);
  const T c2 = S(g.gm1) * (H - S(0.5) * q2);
  const T c = bsqrt(c2);
  const T ic2 = recip(c2);
  // Harten entropy fix (FluxRoe.tpp:158-171)
  const T delta = babs(c * S(g.harten));
  T l1 = babs(vn - c), l2 = babs(vn), l5 = babs(vn + c);
  if (l1 <= delta || l2 <= delta || l5 <= delta) {
    const T ih = S(0.5) * recip(delta);
    if (l1 <= delta) l1 = (l1 * l1 + delta * delta) * ih;
    if (l2 <= delta) l2 = (l2 * l2 + delta * delta) * ih;
    if (l5 <= delta) l5 = (l5 * l5 + delta * delta) * ih;
  }
  const T drho = R.rho - L.rho, dp = R.p - L.p, dvn = R.vn - L.vn;
  T du[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) du[d] = R.u[d] - L.u[d];
  // central part F(UL) + F(UR)
  T FL[5], FR[5];
  euler_flux(UL, L, n, FL);
  euler_flux(UR, R, n, FR);
  const T rc = rho * c;
  // wave 1 (FluxRoe.tpp:174-209)
  const T k1 = l1 * (dp - rc * dvn) * (S(0.5) * ic2);
  // wave 5 (FluxRoe.tpp:269-304)
  const T k5 = l5 * (dp + rc * dvn) * (S(0.5) * ic2);
  // waves 2-4 (FluxRoe.tpp:212-266)
  const T c1 = l2 * (drho - dp * ic2);
  const T cc2 = l2 * rho;
  const T t = du[0] * ua[0] + du[1] * ua[1] + du[2] * ua[2];
  const T k15 = k1 + k5;
  const T k51 = k5 - k1;
  F[0] = S(0.5) * (FL[0] + FR[0] - k15 - c1);
#pragma unroll
  for (int d = 0; d < 3; ++d)
    F[1 + d] = S(0.5) * (FL[1 + d] + FR[1 + d] - k15 * ua[d] - k51 * c * S(n[d]) -
                         (c1 * ua[d] + cc2 * (du[d] - dvn * S(n[d]))));
  F[4] = S(0.5) * (FL[4] + FR[4] - k15 * H - k51 * c * vn -
                   (c1 * S(0.5) * q2 + cc2 * (t - dvn * vn)));
}

// Slip wall (FluxSlipWall_::computeFlux, src/FluxSlipWall.tpp:33-53).
template <class T>
BES_HD void slipwall_flux(const GasConst& g, const T* UL, const double* n, T* F) {
  typedef typename ScalarOf<T>::type S;
  const T k = UL[1] * UL[1] + UL[2] * UL[2] + UL[3] * UL[3];
  const T p = S(g.gm1) * (UL[4] - k * recip(S(2) * UL[0]));
  F[0] = S(0);
  F[1] = p * S(n[0]);
  F[2] = p * S(n[1]);
  F[3] = p * S(n[2]);
  F[4] = S(0);
}

// Euler flux of a primitive boundary state (rho, u, v, w, p, T) (Gas computeAllFlux).
template <class T>
BES_HD void prim_flux(const GasConst& g, const T* P, const double* n, T* F) {
  typedef typename ScalarOf<T>::type S;
  const T vn = P[1] * S(n[0]) + P[2] * S(n[1]) + P[3] * S(n[2]);
  F[0] = P[0] * vn;
  F[1] = P[0] * P[1] * vn + P[4] * S(n[0]);
  F[2] = P[0] * P[2] * vn + P[4] * S(n[1]);
  F[3] = P[0] * P[3] * vn + P[4] * S(n[2]);
  const T vsq = P[1] * P[1] + P[2] * P[2] + P[3] * P[3];
  F[4] = P[0] * (S(g.cp) * P[5] + S(0.5) * vsq) * vn;
}

// Characteristic freestream boundary (FluxFreestream_::computeFlux, src/FluxFreestream.tpp:
// 193-226, branches :35-190).  Pinf = freestream primitives (rho, u, v, w, p, T).
template <class T>
BES_HD void freestream_flux(const GasConst& g, const T* UL, const double* Pinf, const double* n,
                            T* F) {
  typedef typename ScalarOf<T>::type S;
  T P[6];
  const T ir = recip(UL[0]);
  P[0] = UL[0];
  P[1] = UL[1] * ir;
  P[2] = UL[2] * ir;
  P[3] = UL[3] * ir;
  const T k = UL[1] * UL[1] + UL[2] * UL[2] + UL[3] * UL[3];
  const T e = UL[4] - k * (S(0.5) * ir);
  P[4] = S(g.gm1) * e;
  P[5] = e * ir * S(g.inv_cv);
  const T vn = P[1] * S(n[0]) + P[2] * S(n[1]) + P[3] * S(n[2]);
  const T cL = bsqrt(S(g.gamma_R) * P[5]);
  // |vn| / c >= 1  <=>  |vn| >= c  (c > 0)
  const bool super = babs(vn) >= cL;
  if (super && vn <= S(0)) {
    T Pi[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) Pi[i] = S(Pinf[i]);
    prim_flux(g, Pi, n, F);
    return;
  }
  if (super) {
    prim_flux(g, P, n, F);
    return;
  }
  T B[6];
  const T c1 = P[0] * cL;
  const T ic1 = recip(c1);
  const T icl2 = recip(cL * cL);
  if (vn <= S(0)) {  // subsonic inlet (:49-126)
    const T t = S(n[0]) * (S(Pinf[1]) - P[1]) + S(n[1]) * (S(Pinf[2]) - P[2]) +
                S(n[2]) * (S(Pinf[3]) - P[3]);
    B[4] = S(0.5) * (S(Pinf[4]) + P[4] - c1 * t);
    const T c2 = (S(Pinf[4]) - B[4]) * ic1;
    B[0] = S(Pinf[0]) + (B[4] - S(Pinf[4])) * icl2;
#pragma unroll
    for (int d = 0; d < 3; ++d) B[1 + d] = S(Pinf[1 + d]) - c2 * S(n[d]);
  } else {  // subsonic outlet (:129-190)
    B[4] = T(S(Pinf[4]));
    const T c2 = (P[4] - B[4]) * ic1;
    B[0] = P[0] + (B[4] - P[4]) * icl2;
#pragma unroll
    for (int d = 0; d < 3; ++d) B[1 + d] = P[1 + d] + c2 * S(n[d]);
  }
  B[5] = B[4] * recip(S(g.R) * B[0]);
  prim_flux(g, B, n, F);
}

}  // namespace bes
