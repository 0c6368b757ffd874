// Table generation on the GPU: the spherical basis functions from which the
// cylindrical EOF tables are built, evaluated at many points at once.
//
// exptool reads EmpCylSL cache files but cannot build them (eof.py:94-95);
// this project's builder (exptool_gb300/tables/eof_builder.py) constructs
// them from a Sturm-Liouville basis Phi_nl(r) Y_lm(theta): for each azimuthal
// order m it needs, at a disc sample (second-moment matrix) and at every table
// node (tabulation), the functions
//   psi  = Phi_nl Y_lm,   dpsi/dR,   dpsi/dz,   rho_nl Y_lm
// for l = m, m+2, ..., lmax and n < nmax.  One thread per point computes them
// all in FP64: the normalised associated Legendre recurrence of this m (kept
// two terms at a time), the theta derivative, and the radial functions from
// the cubic-spline coefficients of u_nl(ln r) (Phi_nl = u Phi0 / sqrt(mu),
// 4 pi rho_nl = u 4 pi rho0 sqrt(mu)).  The products with the eigenvectors
// are plain FP64 GEMMs done by the caller.
#include "xt_internal.cuh"

namespace xt {

struct EofBasisArgs {
  int m, lmax, nmax, nseg;
  const double* knots;      // [nseg + 1] spline breakpoints in t = ln r (ascending)
  const double* coef;       // [lmax + 1][nseg][nmax][4], descending powers of (t - knot)
  const double* inv_sqrt_ev, *sqrt_ev;   // [lmax + 1][nmax]
  const double *R, *z, *phi0, *dphi0, *rho0;   // [npt]; the model at r = max(sqrt(R^2 + z^2), rmin)
  double rmin;
  long long npt;
  int derivs;
  double *psi, *dR, *dz, *rho;   // [nfunc][npt]
};

__global__ void __launch_bounds__(128) k_eof_basis(EofBasisArgs a) {
  const double inv4pi = 1.0 / (4.0 * 3.14159265358979323846);
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < a.npt;
       p += (long long)gridDim.x * blockDim.x) {
    const double R = a.R[p], z = a.z[p];
    double r = sqrt(R * R + z * z);
    if (r < a.rmin) r = a.rmin;
    const double c = z / r;
    const double s = sqrt(fmax(0.0, (1.0 - c) * (1.0 + c)));
    const double t = log(r);
    // spline interval (extrapolation beyond the ends uses the end intervals)
    int lo = 0, hi = a.nseg;                     // knots[lo] <= t < knots[hi]
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (t >= a.knots[mid]) lo = mid;
      else hi = mid;
    }
    const double dx = t - a.knots[lo];
    const double ph = a.phi0[p], dph = a.dphi0[p], rh = a.rho0[p];
    const double m2 = (double)a.m * a.m;
    // normalised sectoral term N_mm P_mm with the Condon-Shortley phase
    double ymm = sqrt(inv4pi);
    for (int k = 1; k <= a.m; ++k) ymm = -sqrt((2.0 * k + 1.0) / (2.0 * k)) * s * ymm;
    const double sq2 = a.m > 0 ? sqrt(2.0) : 1.0;
    double y2 = 0.0, y1 = ymm;                   // Y[l-2], Y[l-1] before the l loop (unscaled)
    const bool safe = s > 1e-12;
    int f = 0;
    for (int l = a.m; l <= a.lmax; ++l) {
      double yl;
      if (l == a.m) yl = ymm;
      else if (l == a.m + 1) yl = sqrt(2.0 * a.m + 3.0) * c * ymm;
      else {
        const double A = sqrt((4.0 * l * l - 1.0) / (l * l - m2));
        const double B = sqrt(((l - 1.0) * (l - 1.0) - m2) / (4.0 * (l - 1.0) * (l - 1.0) - 1.0));
        yl = A * (c * y1 - B * y2);
      }
      if (l > a.m) {
        y2 = y1;
        y1 = yl;
      }
      if (((l - a.m) & 1) == 0) {
        const double Y = sq2 * yl;
        double dY = 0.0;
        if (a.derivs && safe) {
          const double yprev = l > a.m ? sq2 * y2 : 0.0;
          const double cf = l > a.m ? sqrt((2.0 * l + 1.0) / (2.0 * l - 1.0) * (l * l - m2)) : 0.0;
          dY = (l * c * Y - cf * yprev) / s;
        }
        const double* cl = a.coef + ((size_t)l * a.nseg + lo) * a.nmax * 4;
        for (int n = 0; n < a.nmax; ++n, ++f) {
          const double* q = cl + 4 * n;
          const double u = ((q[0] * dx + q[1]) * dx + q[2]) * dx + q[3];
          const double ie = a.inv_sqrt_ev[l * a.nmax + n];
          const double pot = u * ph * ie;
          const size_t o = (size_t)f * a.npt + p;
          a.psi[o] = pot * Y;
          if (a.derivs) {
            const double du = (3.0 * q[0] * dx + 2.0 * q[1]) * dx + q[2];
            const double dpot = (du * ph / r + u * dph) * ie;
            a.dR[o] = dpot * (R / r) * Y + pot * dY * (z / (r * r));
            a.dz[o] = dpot * (z / r) * Y - pot * dY * (R / (r * r));
            a.rho[o] = u * rh * a.sqrt_ev[l * a.nmax + n] * Y;
          }
        }
      }
    }
  }
}

}  // namespace xt

using namespace xt;

extern "C" {

int xt_eof_basis(int m, int lmax, int nmax, int nseg, const double* knots, const double* coef,
                 const double* inv_sqrt_ev, const double* sqrt_ev, const double* R, const double* z,
                 const double* phi0, const double* dphi0, const double* rho0, double rmin, long long npt, int derivs,
                 double* psi, double* dR, double* dz, double* rho, void* stream) {
  XT_REQUIRE(m >= 0 && lmax >= m && nmax >= 1 && nseg >= 1, "bad basis sizes (m %d, lmax %d, nmax %d, nseg %d)", m,
             lmax, nmax, nseg);
  XT_REQUIRE(npt >= 0, "negative point count");
  if (npt == 0) return XT_OK;
  XT_REQUIRE(knots && coef && inv_sqrt_ev && sqrt_ev && R && z && phi0 && dphi0 && rho0 && psi, "NULL array");
  XT_REQUIRE(!derivs || (dR && dz && rho), "NULL derivative or density output");
  EofBasisArgs a{m, lmax, nmax, nseg, knots, coef, inv_sqrt_ev, sqrt_ev, R, z, phi0, dphi0, rho0, rmin, npt,
                 derivs ? 1 : 0, psi, dR, dz, rho};
  k_eof_basis<<<grid_for(npt, 128, 8), 128, 0, as_stream(stream)>>>(a);
  XT_CHECK_LAUNCH("k_eof_basis");
  return XT_OK;
}

}  // extern "C"
