// hbi_rsf.cuh -- the rate-and-state friction derivative (deriv,
// main_LH.f90:2165-2244) and the slip rate of a state, shared by the
// single-system epilogue (hbi_matvec.cu) and the ensemble (hbi_ens.cu).
// `Law` provides evlaw, limitsigma, vref, minsig, maxsig, rigid_over_2vs.
#pragma once

namespace hbi {

// slip rate V = 2 vref e^(-psi/a) sinh(s) and W = 2 vref e^(-psi/a) cosh(s),
// s = tau/(sigma a) (main_LH.f90:1277 and the dV/dtau factor of :2165-2244),
// with one exponential: for |s| > 1, 2 e^(-psi/a) sinh(s) = sign(s) e^(|s| -
// psi/a) (1 - e^(-2|s|)) and likewise for cosh with (1 + e^(-2|s|)); e^(-2|s|)
// is below double resolution for |s| >= 20 (friction / a is about 60 here).
__device__ __forceinline__ void slip_rate_w(double vref, double psi, double tau, double sig, double a, double* V,
                                            double* W) {
  const double s = tau / sig / a;
  const double q = -psi / a;
  const double as = fabs(s);
  if (as > 1.0) {
    const double E = exp(q + as);
    const double r = as < 20.0 ? exp(-2.0 * as) : 0.0;
    *V = copysign(vref * E * (1.0 - r), s);
    *W = vref * E * (1.0 + r);
  } else {
    const double e = exp(q);
    *V = 2 * vref * e * sinh(s);
    *W = 2 * vref * e * cosh(s);
  }
}

__device__ __forceinline__ double slip_rate(double vref, double psi, double tau, double sig, double a) {
  double v, w;
  slip_rate_w(vref, psi, tau, sig, a, &v, &w);
  return v;
}

// deriv (main_LH.f90:2165-2244): aging (0) and slip (1) laws; vel and w are
// the state's V and W (slip_rate_w)
template <typename Law>
__device__ __forceinline__ void deriv_dev(const Law& R, double sum_gs, double sum_gn, double psi, double tau,
                                          double sig, double vel, double w, double a, double b, double dc, double f0,
                                          double* out) {
  double dsig = sum_gn;
  if (R.limitsigma) {
    if (sig < R.minsig) dsig = 0;
    if (sig > R.maxsig) dsig = 0;
  }
  const double vref = R.vref;
  double dpsi;
  if (R.evlaw == 0) {
    dpsi = (b == 0) ? 0.0 : b / dc * vref * exp((f0 - psi) / b) - b * fabs(vel) / dc;
  } else {
    const double fss = f0 + (a - b) * log(fabs(vel) / vref);
    dpsi = -(fabs(vel) / dc * (fabs(tau) / sig - fss));
  }
  const double dvdtau = w / (a * sig);
  const double dvdsig = -(w * tau / (a * (sig * sig)));
  const double dvdpsi = -vel / a;
  const double t = sum_gs - R.rigid_over_2vs * (dvdpsi * dpsi + dvdsig * dsig);
  out[0] = dpsi;
  out[1] = t / (1.0 + R.rigid_over_2vs * dvdtau);
  out[2] = dsig;
}

}  // namespace hbi
