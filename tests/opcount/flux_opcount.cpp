// Floating-point operation counts of the face fluxes, per face, by instantiating the same
// templates the GPU kernels use (bes_gb300/csrc/physics.cuh) with a counting scalar: each
// add/sub, mul, division (reciprocal), square root, |x| and comparison of two values is
// counted once.  Test infrastructure: prints one JSON object per flux branch.
#include <cstdio>

struct Counts {
  long add = 0, mul = 0, div = 0, sqrt = 0, abs = 0, cmp = 0;
};
static Counts g_c;

struct Cnt {
  double v;
  Cnt() : v(0) {}
  Cnt(double x) : v(x) {}  // NOLINT: constants of the templates
};
inline Cnt operator+(Cnt a, Cnt b) { ++g_c.add; return Cnt(a.v + b.v); }
inline Cnt operator-(Cnt a, Cnt b) { ++g_c.add; return Cnt(a.v - b.v); }
inline Cnt operator*(Cnt a, Cnt b) { ++g_c.mul; return Cnt(a.v * b.v); }
inline Cnt operator/(Cnt a, Cnt b) { ++g_c.div; return Cnt(a.v / b.v); }
inline Cnt operator-(Cnt a) { return Cnt(-a.v); }  // a sign flip, folded into the consumer
inline Cnt& operator+=(Cnt& a, Cnt b) { a = a + b; return a; }
inline Cnt& operator-=(Cnt& a, Cnt b) { a = a - b; return a; }
inline Cnt& operator*=(Cnt& a, Cnt b) { a = a * b; return a; }
inline bool operator<=(Cnt a, Cnt b) { ++g_c.cmp; return a.v <= b.v; }
inline bool operator>=(Cnt a, Cnt b) { ++g_c.cmp; return a.v >= b.v; }
inline bool operator<(Cnt a, Cnt b) { ++g_c.cmp; return a.v < b.v; }
inline bool operator>(Cnt a, Cnt b) { ++g_c.cmp; return a.v > b.v; }
Cnt recip(Cnt a);
Cnt bsqrt(Cnt a);
Cnt babs(Cnt a);

#include "../../bes_gb300/csrc/physics.cuh"

#include <cmath>
Cnt recip(Cnt a) { ++g_c.div; return Cnt(1.0 / a.v); }
Cnt bsqrt(Cnt a) { ++g_c.sqrt; return Cnt(std::sqrt(a.v)); }
Cnt babs(Cnt a) { ++g_c.abs; return Cnt(std::fabs(a.v)); }

static void cons(double rho, double u, double v, double w, double p, double gamma, Cnt* U) {
  U[0] = rho;
  U[1] = rho * u;
  U[2] = rho * v;
  U[3] = rho * w;
  U[4] = p / (gamma - 1.0) + 0.5 * rho * (u * u + v * v + w * w);
}

static void report(const char* name) {
  std::printf("{\"flux\": \"%s\", \"add\": %ld, \"mul\": %ld, \"div\": %ld, \"sqrt\": %ld, "
              "\"abs\": %ld, \"cmp\": %ld}\n",
              name, g_c.add, g_c.mul, g_c.div, g_c.sqrt, g_c.abs, g_c.cmp);
  g_c = Counts();
}

int main() {
  const double gamma = 1.4, R = 287.0;
  const bes::GasConst g = bes::make_gas(R, gamma, 0.05);
  const double n[3] = {0.6, 0.8, 0.0};
  Cnt UL[5], UR[5], F[5];
  // Roe, no wave inside Harten's band
  cons(1.0, 0.5, 0.1, 0.0, 1.0 / gamma, gamma, UL);
  cons(1.05, 0.45, 0.12, 0.01, 1.02 / gamma, gamma, UR);
  g_c = Counts();
  bes::roe_flux(g, UL, UR, n, F);
  report("roe");
  // Roe, the normal velocity inside the band (one wave corrected)
  cons(1.0, 0.01, -0.0075, 0.0, 1.0 / gamma, gamma, UL);
  cons(1.0, 0.012, -0.009, 0.0, 1.0 / gamma, gamma, UR);
  g_c = Counts();
  bes::roe_flux(g, UL, UR, n, F);
  report("roe_harten_one_wave");
  g_c = Counts();
  bes::slipwall_flux(g, UL, n, F);
  report("slip_wall");
  const double Pinf[6] = {1.0, 0.5, 0.0, 0.0, 1.0 / gamma, 1.0 / (gamma * R)};
  // freestream branches: subsonic inlet, subsonic outlet, supersonic inlet, supersonic outlet
  const double vel[4][3] = {{-0.5, 0, 0}, {0.5, 0, 0}, {-2.0, 0, 0}, {2.0, 0, 0}};
  const char* names[4] = {"freestream_subsonic_in", "freestream_subsonic_out",
                          "freestream_supersonic_in", "freestream_supersonic_out"};
  const double nx[3] = {1.0, 0.0, 0.0};
  for (int b = 0; b < 4; ++b) {
    cons(1.0, vel[b][0], vel[b][1], vel[b][2], 1.0 / gamma, gamma, UL);
    g_c = Counts();
    bes::freestream_flux(g, UL, Pinf, nx, F);
    report(names[b]);
  }
  return 0;
}
