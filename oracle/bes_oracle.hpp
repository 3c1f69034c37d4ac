// CPU restatement of joel-ho/BES's steady residual/update path.
// TEST INFRASTRUCTURE ONLY: the checker for the GPU library (tests, smoke() and the
// bench's CPU-baseline leg use it); the product never links or calls it.
//
// Parity pin: golden binaries produced by the reference itself (oracle/ref, built from the
// reference sources) are committed under tests/golden/ and this restatement is checked
// against them.  Operation order follows the reference so that, compiled without FMA
// contraction, most quantities agree bit for bit.
//
// Each function cites the reference file:line it restates.
#pragma once
#include <cmath>
#include <cstdint>
#include <vector>

namespace bor {

// ---------------------------------------------------------------------------------
// Forward-mode dual numbers (the reference differentiates its flux templates with
// Eigen::AutoDiffScalar, src/FluxJacobianWrapper.tpp:32-82).
// ---------------------------------------------------------------------------------
template <int N>
struct Dual {
  double v;
  double d[N];
  Dual() : v(0.0) {
    for (int i = 0; i < N; ++i) d[i] = 0.0;
  }
  Dual(double x) : v(x) {  // NOLINT: implicit like AutoDiffScalar
    for (int i = 0; i < N; ++i) d[i] = 0.0;
  }
};
template <int N> inline Dual<N> operator+(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r(a.v + b.v);
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] + b.d[i];
  return r;
}
template <int N> inline Dual<N> operator-(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r(a.v - b.v);
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] - b.d[i];
  return r;
}
template <int N> inline Dual<N> operator-(const Dual<N>& a) {
  Dual<N> r(-a.v);
  for (int i = 0; i < N; ++i) r.d[i] = -a.d[i];
  return r;
}
template <int N> inline Dual<N> operator*(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r(a.v * b.v);
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
  return r;
}
template <int N> inline Dual<N> operator/(const Dual<N>& a, const Dual<N>& b) {
  Dual<N> r(a.v / b.v);
  const double ib = 1.0 / b.v;
  for (int i = 0; i < N; ++i) r.d[i] = (a.d[i] - r.v * b.d[i]) * ib;
  return r;
}
template <int N> inline Dual<N> operator+(const Dual<N>& a, double b) { return a + Dual<N>(b); }
template <int N> inline Dual<N> operator+(double a, const Dual<N>& b) { return Dual<N>(a) + b; }
template <int N> inline Dual<N> operator-(const Dual<N>& a, double b) { return a - Dual<N>(b); }
template <int N> inline Dual<N> operator-(double a, const Dual<N>& b) { return Dual<N>(a) - b; }
template <int N> inline Dual<N> operator*(const Dual<N>& a, double b) {
  Dual<N> r(a.v * b);
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * b;
  return r;
}
template <int N> inline Dual<N> operator*(double a, const Dual<N>& b) {
  Dual<N> r(a * b.v);
  for (int i = 0; i < N; ++i) r.d[i] = a * b.d[i];
  return r;
}
template <int N> inline Dual<N> operator/(const Dual<N>& a, double b) {
  Dual<N> r(a.v / b);
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] / b;
  return r;
}
template <int N> inline Dual<N> operator/(double a, const Dual<N>& b) { return Dual<N>(a) / b; }
template <int N> inline Dual<N>& operator+=(Dual<N>& a, const Dual<N>& b) { return a = a + b; }
template <int N> inline Dual<N>& operator-=(Dual<N>& a, const Dual<N>& b) { return a = a - b; }
template <int N> inline Dual<N>& operator/=(Dual<N>& a, double b) { return a = a / b; }
template <int N> inline Dual<N> sqrt(const Dual<N>& a) {
  Dual<N> r(std::sqrt(a.v));
  const double h = 0.5 / r.v;
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * h;
  return r;
}
template <int N> inline Dual<N> abs(const Dual<N>& a) {
  Dual<N> r(std::fabs(a.v));
  const double s = a.v < 0 ? -1.0 : 1.0;
  for (int i = 0; i < N; ++i) r.d[i] = a.d[i] * s;
  return r;
}
template <int N> inline bool operator>(const Dual<N>& a, const Dual<N>& b) { return a.v > b.v; }
template <int N> inline bool operator>(const Dual<N>& a, double b) { return a.v > b; }
template <int N> inline bool operator>=(const Dual<N>& a, double b) { return a.v >= b; }
template <int N> inline bool operator<(const Dual<N>& a, double b) { return a.v < b; }
template <int N> inline bool operator<=(const Dual<N>& a, double b) { return a.v <= b; }
inline double value_of(double x) { return x; }
template <int N> inline double value_of(const Dual<N>& x) { return x.v; }
using std::abs;
using std::sqrt;

// ---------------------------------------------------------------------------------
// Gas: perfect gas, non-dimensional Euler, 3-D (src/GasPerfect.tpp:22-328, src/Gas.tpp:30-87)
// Conserved U = (rho, rho u, rho v, rho w, rho E); primitive P = (rho, u, v, w, p, T).
// ---------------------------------------------------------------------------------
struct Gas {
  double R = 287.0, gamma = 1.4, cv = 0, cp = 0;
  void init(double gas_constant, double ratio) {  // GasPerfect.tpp:22-28
    R = gas_constant;
    gamma = ratio;
    cv = R / (gamma - 1.0);
    cp = cv + R;
  }
  template <class T> T kinetic2(const T* U) const {  // sum (rho u_d)^2
    T s = 0.0;
    for (int d = 0; d < 3; ++d) s += U[1 + d] * U[1 + d];
    return s;
  }
  template <class T> T pressure(const T* U) const {  // GasPerfect.tpp:48-64
    return (gamma - 1.0) * (U[4] - kinetic2(U) / (2.0 * U[0]));
  }
  template <class T> T temperature(const T* U) const {  // GasPerfect.tpp:67-85
    return (1.0 / (cv * U[0])) * (U[4] - kinetic2(U) / (2.0 * U[0]));
  }
  template <class T> T velocity(const T* U, int d) const { return U[1 + d] / U[0]; }
  template <class T> void primitive(const T* U, T* P) const {  // GasPerfect.tpp:88-112
    P[0] = U[0];
    for (int d = 0; d < 3; ++d) P[1 + d] = velocity(U, d);
    P[4] = pressure(U);
    P[5] = temperature(U);
  }
  template <class T> T velocity_sq(const T* U) const {  // GasPerfect.tpp:119-131
    T s = 0.0;
    for (int d = 0; d < 3; ++d) s += velocity(U, d) * velocity(U, d);
    return s;
  }
  template <class T> T total_enthalpy(const T* U) const {  // GasPerfect.tpp:133-146
    return U[4] / U[0] + pressure(U) / U[0];
  }
  template <class T> T sound_speed_T(const T& temp) const {  // GasPerfect.tpp:149-151
    return sqrt(gamma * R * temp);
  }
  // Q3: sqrt(gamma (gamma-1) (H - q^2/2)) = sqrt(gamma) * true c (GasPerfect.tpp:154-160)
  template <class T> T sound_speed_U(const T* U) const {
    return sqrt(gamma * (gamma - 1.0) * (total_enthalpy(U) - velocity_sq(U) / 2.0));
  }
  template <class T> T contravariant_U(const T* U, const double* n) const {  // :163-174
    T s = 0.0;
    for (int d = 0; d < 3; ++d) s += velocity(U, d) * n[d];
    return s;
  }
  template <class T> T contravariant_P(const T* P, const double* n) const {  // Gas.tpp:30-41
    T s = 0.0;
    for (int d = 0; d < 3; ++d) s += P[1 + d] * n[d];
    return s;
  }
  template <class T> void conserved(const T* P, T* U) const {  // GasPerfect.tpp:182-216
    U[0] = P[0];
    T s = 0.0;
    for (int d = 0; d < 3; ++d) {
      U[1 + d] = U[0] * P[1 + d];
      s += P[1 + d] * P[1 + d];
    }
    U[4] = U[0] * (cv * P[5] + s / 2.0);
  }
  template <class T> void flux_P(const T* P, const double* n, T* F) const {  // :266-291
    const T vn = contravariant_P(P, n);
    F[0] = P[0] * vn;
    for (int d = 0; d < 3; ++d) F[1 + d] = P[0] * P[1 + d] * vn + P[4] * n[d];
    T vsq = 0.0;
    for (int d = 0; d < 3; ++d) vsq += P[1 + d] * P[1 + d];
    F[4] = P[0] * (cp * P[5] + vsq / 2.0) * vn;
  }
};

// Roe flux-difference splitting with Harten's entropy fix (src/FluxRoe.tpp:21-333).
template <class T>
void flux_roe(const Gas& g, double harten, const T* UL, const T* UR, const double* n, T* F) {
  // per-side variables: rho u v w p T H C Vn q2   (FluxRoe.tpp:61-76)
  T L[10], R[10], D[10], A[10];
  auto side = [&](const T* U, T* P) {
    g.primitive(U, P);
    P[6] = g.total_enthalpy(U);
    P[7] = g.sound_speed_U(U);
    P[8] = g.contravariant_U(U, n);
    P[9] = g.velocity_sq(U);
  };
  side(UL, L);
  side(UR, R);
  for (int i = 0; i < 10; ++i) D[i] = R[i] - L[i];
  // Roe averages (FluxRoe.tpp:110-143)
  const T den = sqrt(L[0]) + sqrt(R[0]);
  A[9] = 0.0;
  A[8] = 0.0;
  A[0] = sqrt(L[0] * R[0]);
  for (int d = 0; d < 3; ++d) {
    A[1 + d] = (L[1 + d] * sqrt(L[0]) + R[1 + d] * sqrt(R[0])) / den;
    A[9] += A[1 + d] * A[1 + d];
    A[8] += A[1 + d] * n[d];
  }
  A[6] = (L[6] * sqrt(L[0]) + R[6] * sqrt(R[0])) / den;
  A[7] = sqrt((g.gamma - 1.0) * (A[6] - A[9] / 2.0));
  auto harten_fix = [&](const T& lam) -> T {  // FluxRoe.tpp:158-171
    const T delta = abs(A[7] * harten);
    if (lam > delta) return lam;
    return (lam * lam + delta * delta) / (2.0 * delta);
  };
  T tmp[5];
  for (int i = 0; i < 5; ++i) F[i] = 0.0;
  g.flux_P(L, n, tmp);  // FluxRoe.tpp:146-155
  for (int i = 0; i < 5; ++i) F[i] += tmp[i];
  g.flux_P(R, n, tmp);
  for (int i = 0; i < 5; ++i) F[i] += tmp[i];
  {  // wave 1 (FluxRoe.tpp:174-209)
    const T c = harten_fix(abs(A[8] - A[7])) * (D[4] - A[0] * A[7] * D[8]) / (2.0 * A[7] * A[7]);
    F[0] -= c;
    for (int d = 0; d < 3; ++d) F[1 + d] -= c * (A[1 + d] - A[7] * n[d]);
    F[4] -= c * (A[6] - A[7] * A[8]);
  }
  {  // waves 2-4 (FluxRoe.tpp:212-266)
    T t = 0.0;
    const T lam = harten_fix(abs(A[8]));
    const T c1 = lam * (D[0] - D[4] / (A[7] * A[7]));
    const T c2 = lam * A[0];
    F[0] -= c1;
    for (int d = 0; d < 3; ++d) {
      F[1 + d] -= (c1 * A[1 + d] + c2 * (D[1 + d] - D[8] * n[d]));
      t += D[1 + d] * A[1 + d];
    }
    F[4] -= (c1 * A[9] / 2.0 + c2 * (t - D[8] * A[8]));
  }
  {  // wave 5 (FluxRoe.tpp:269-304)
    const T c = harten_fix(abs(A[8] + A[7])) * (D[4] + A[0] * A[7] * D[8]) / (2.0 * A[7] * A[7]);
    F[0] -= c;
    for (int d = 0; d < 3; ++d) F[1 + d] -= c * (A[1 + d] + A[7] * n[d]);
    F[4] -= c * (A[6] + A[7] * A[8]);
  }
  for (int i = 0; i < 5; ++i) F[i] /= 2.0;
}

// Characteristic freestream boundary (src/FluxFreestream.tpp:35-226).  Pinf is the
// freestream PRIMITIVE vector (rho, u, v, w, p, T).
template <class T>
void flux_freestream(const Gas& g, const T* UL, const double* Pinf_d, const double* n, T* F) {
  T L[6], Pinf[6], B[6];
  for (int i = 0; i < 6; ++i) Pinf[i] = Pinf_d[i];
  g.primitive(UL, L);
  const T vn = g.contravariant_P(L, n);
  const T mach = abs(vn) / g.sound_speed_T(L[5]);
  if (mach >= 1.0 && vn <= 0.0) {
    g.flux_P(Pinf, n, F);  // supersonic inlet :35-39
  } else if (mach >= 1.0 && vn > 0.0) {
    g.flux_P(L, n, F);  // supersonic outlet :42-46
  } else if (mach < 1.0 && vn <= 0.0) {  // subsonic inlet :49-126
    const T cL = g.sound_speed_T(L[5]);
    T t = 0.0;
    for (int d = 0; d < 3; ++d) t += n[d] * (Pinf[1 + d] - L[1 + d]);
    const T c1 = L[0] * cL;
    B[4] = (Pinf[4] + L[4] - c1 * t) / 2.0;
    const T c2 = (Pinf[4] - B[4]) / c1;
    B[0] = Pinf[0] + (B[4] - Pinf[4]) / (cL * cL);
    B[5] = B[4] / (g.R * B[0]);
    for (int d = 0; d < 3; ++d) B[1 + d] = Pinf[1 + d] - c2 * n[d];
    g.flux_P(B, n, F);
  } else if (mach < 1.0 && vn > 0.0) {  // subsonic outlet :129-190
    const T cL = g.sound_speed_T(L[5]);
    const T c1 = L[0] * cL;
    B[4] = Pinf[4];
    const T c2 = (L[4] - B[4]) / c1;
    B[0] = L[0] + (B[4] - L[4]) / (cL * cL);
    B[5] = B[4] / (g.R * B[0]);
    for (int d = 0; d < 3; ++d) B[1 + d] = L[1 + d] + c2 * n[d];
    g.flux_P(B, n, F);
  }
}

// Slip wall: pressure only (src/FluxSlipWall.tpp:33-53).
template <class T>
void flux_slipwall(const Gas& g, const T* UL, const double* n, T* F) {
  for (int i = 0; i < 5; ++i) F[i] = 0.0;
  const T p = g.pressure(UL);
  for (int d = 0; d < 3; ++d) F[1 + d] = p * n[d];
}

enum FaceKind { FACE_INTERNAL = 0, FACE_SLIP_WALL = 1, FACE_FREESTREAM = 2 };

// Reference-semantics mesh (src/Mesh.cpp:95-636, src/MeshGmsh.cpp, src/Element.cpp).
struct Mesh {
  int64_t nc = 0, nf = 0;
  int dim = 3;  // 2: triangles, edges as faces, z ignored
  int nfc = 4;  // faces per cell (3 for triangles: local slot 3 is empty, cface = cadj = -1)
  // faces in reference creation order
  std::vector<double> S, nhat, area, center;  // [nf*3], [nf*3], [nf], [nf*3]
  std::vector<int64_t> owner, neigh;          // neigh = -1 on boundary
  std::vector<int> kind;
  // cells in file order
  std::vector<double> vol, centroid;  // [nc], [nc*3]
  std::vector<int64_t> cface, cadj;   // [nc*4]: face id and adjacent cell (-1) per local face
  std::vector<double> weight, rvec;   // [nc*4], [nc*12]
  std::vector<double> plen;           // projected lengths [nc*3] (TimeStepCalculatorLocal.cpp:51-65)
  std::vector<int> muscl_slot;        // [nc*4] local face whose vector MUSCL uses
};

struct Options {
  int solver = 0;  // 0 explicit, 1 implicit
  int local_dt = 1;
  double cfl = 0.8;
  double cfl_max = 0.0;  // adaptive CFL active when cfl_max > cfl
  double cfl_exp[2] = {1.0, 1.0};
  int n_stage = 4;
  double alpha[8] = {0.0833, 0.2069, 0.4265, 1.0, 0, 0, 0, 0};
  double venkat_k = 5.0;
  double harten = 0.05;
  double gas_constant = 287.0;
  double gamma = 1.4;
  double mach[3] = {0.5, 0.0, 0.0};
  int muscl_exact = 0;     // 0: reproduce the reference's face-vector lookup (quirk Q13)
  int jacobian_repeat = 5;  // Q9: blocks added once per conserved variable
  int lin_precond = 0;      // 0 block Jacobi, 1 block ILU(0)
  int lin_restart = 30;
  int lin_maxiter = 1000;
  double lin_tol = 1e-7;
  // CFL ramp (new, additive): if ramp_steps > 0, CFL_k = cfl0 * (cfl1/cfl0)^(k/(ramp_steps-1))
  int ramp_steps = 0;
  double ramp_cfl0 = 0.0, ramp_cfl1 = 0.0;
  int fs_ramp = 0;          // FREESTREAM_RAMP
  double fs_frac = 0.5;     // FREESTREAM_RAMP_START_FRAC
};

}  // namespace bor
