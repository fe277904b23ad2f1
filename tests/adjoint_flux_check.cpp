// Host check of the hand-written reverse-mode flux derivatives (rusanov_vjp, hllc_vjp,
// roe_vjp, composed with prim_r and prim_vjp) against forward-mode dual numbers through the
// flux templates of the residual's operation order.  Random conservative states (subsonic,
// transonic, supersonic, nearly equal left/right), random unit normals and random adjoint
// weights.  Prints one line per scheme:
//   <scheme> <cases> <max relative error> <cases per flux branch ...>
#include <cmath>
#include <cstdio>
#include <random>

#include "../typhon_gb300/csrc/adjoint_flux.cuh"

using namespace tyk::adflux;

namespace {

struct Case {
  double uL[5], uR[5], n[3], Fb[5];
};

Case make_case(std::mt19937_64& r, int it) {
  std::uniform_real_distribution<double> U(-1.0, 1.0);
  Case c;
  const double vmax = (it % 3 == 0) ? 0.3 : (it % 3 == 1 ? 1.5 : 4.0);
  double* st[2] = {c.uL, c.uR};
  for (double* u : st) {
    u[0] = 1.0 + 0.5 * U(r);
    for (int k = 2; k < 5; ++k) u[k] = u[0] * vmax * U(r);
    const double p = 1.0 + 0.5 * U(r);
    u[1] = p / 0.4 + 0.5 * (u[2] * u[2] + u[3] * u[3] + u[4] * u[4]) / u[0];
  }
  if (it % 7 == 0)
    for (int v = 0; v < 5; ++v) c.uR[v] = c.uL[v] * (1.0 + 1e-3 * U(r));
  double nn = 0.0;
  for (double& x : c.n) { x = U(r); nn += x * x; }
  for (double& x : c.n) x /= std::sqrt(nn);
  for (double& x : c.Fb) x = U(r);
  return c;
}

// (dF/dU_L)^T Fb and (dF/dU_R)^T Fb by dual numbers (ref) and by the hand-written reverse (got)
template <int SCH>
double check(const Case& c, double g, double eps) {
  double ref[10];
  for (int side = 0; side < 2; ++side) {
    Dual<5> UL[5], UR[5], QL[5], QR[5], F[5];
    for (int v = 0; v < 5; ++v) {
      UL[v] = Dual<5>(c.uL[v]);
      UR[v] = Dual<5>(c.uR[v]);
      (side == 0 ? UL : UR)[v].d[v] = 1.0;
    }
    prim_t(g, UL, QL);
    prim_t(g, UR, QR);
    if (SCH == 0) flux_rusanov_t(g, QL, QR, c.n[0], c.n[1], c.n[2], F);
    else if (SCH == 1) flux_hllc_t(g, QL, QR, c.n[0], c.n[1], c.n[2], F);
    else flux_roe_t(g, eps, QL, QR, c.n[0], c.n[1], c.n[2], F);
    for (int j = 0; j < 5; ++j) {
      double s = 0.0;
      for (int v = 0; v < 5; ++v) s += c.Fb[v] * F[v].d[j];
      ref[5 * side + j] = s;
    }
  }
  double QL[5], QR[5], QLb[5] = {0, 0, 0, 0, 0}, QRb[5] = {0, 0, 0, 0, 0};
  double got[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  const double irL = prim_r(g, c.uL, QL), irR = prim_r(g, c.uR, QR);
  if (SCH == 0) rusanov_vjp(g, QL, QR, c.n[0], c.n[1], c.n[2], c.Fb, QLb, QRb);
  else if (SCH == 1) hllc_vjp(g, QL, QR, c.n[0], c.n[1], c.n[2], c.Fb, QLb, QRb);
  else roe_vjp(g, eps, QL, QR, c.n[0], c.n[1], c.n[2], c.Fb, QLb, QRb);
  prim_vjp(g, c.uL, irL, QLb, got);
  prim_vjp(g, c.uR, irR, QRb, got + 5);
  double sc = 0.0, err = 0.0;
  for (int j = 0; j < 10; ++j) sc = std::fmax(sc, std::fabs(ref[j]));
  for (int j = 0; j < 10; ++j) err = std::fmax(err, std::fabs(got[j] - ref[j]));
  return sc > 0.0 ? err / sc : err;
}

// which branch of the flux a case takes (for the coverage counts)
int branch(int sch, const Case& c, double g, double eps) {
  double QL[5], QR[5];
  prim_t(g, c.uL, QL);
  prim_t(g, c.uR, QR);
  const double* L = QL;
  const double* R = QR;
  const double vnl = L[2] * c.n[0] + L[3] * c.n[1] + L[4] * c.n[2];
  const double vnr = R[2] * c.n[0] + R[3] * c.n[1] + R[4] * c.n[2];
  const double al = std::sqrt(g * L[1] / L[0]), ar = std::sqrt(g * R[1] / R[0]);
  if (sch == 0) return std::fabs(vnr) + ar > std::fabs(vnl) + al ? 1 : 0;
  if (sch == 1) {
    // the HLLC estimates reduce to sign tests of the exact-flux kernel; count by the left and
    // right wave bounds of the simple Davis estimate, close enough for coverage
    if (vnl - al >= 0.0) return 0;
    if (vnr + ar <= 0.0) return 1;
    return 2;
  }
  const double vn = 0.5 * (vnl + vnr), a = 0.5 * (al + ar);
  return (std::fabs(vn - a) < eps * a || std::fabs(vn + a) < eps * a) ? 1 : 0;
}

}  // namespace

int main() {
  const double g = 1.4;
  const char* names[3] = {"RUSANOV", "HLLC", "ROE"};
  for (int sch = 0; sch < 3; ++sch) {
    std::mt19937_64 r(1234 + sch);
    const int ncase = 30000;
    double worst = 0.0;
    int hits[3] = {0, 0, 0};
    for (int it = 0; it < ncase; ++it) {
      const Case c = make_case(r, it);
      const double eps = (it & 1) ? 0.1 : 0.6;
      double e = sch == 0 ? check<0>(c, g, eps) : (sch == 1 ? check<1>(c, g, eps) : check<2>(c, g, eps));
      worst = std::fmax(worst, e);
      hits[branch(sch, c, g, eps)]++;
    }
    std::printf("%s %d %.3e %d %d %d\n", names[sch], ncase, worst, hits[0], hits[1], hits[2]);
  }
  return 0;
}
