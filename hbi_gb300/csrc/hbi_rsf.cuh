// hbi_rsf.cuh -- the rate-and-state friction derivative (deriv,
// main_LH.f90:2165-2244) and the slip rate of a state, shared by the
// single-system epilogue (hbi_matvec.cu) and the ensemble (hbi_ens.cu).
// `Law` provides evlaw, limitsigma, vref, minsig, maxsig, rigid_over_2vs.
#pragma once

namespace hbi {

// deriv (main_LH.f90:2165-2244): aging (0) and slip (1) laws
template <typename Law>
__device__ __forceinline__ void deriv_dev(const Law& R, double sum_gs, double sum_gn, double psi, double tau,
                                          double sig, double vel, double a, double b, double dc, double f0,
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
  const double e = exp(-psi / a), ch = cosh(tau / sig / a);
  const double dvdtau = 2 * vref * e * ch / (a * sig);
  const double dvdsig = -(2 * vref * e * ch * tau / (a * (sig * sig)));
  const double dvdpsi = -vel / a;
  const double t = sum_gs - R.rigid_over_2vs * (dvdpsi * dpsi + dvdsig * dsig);
  out[0] = dpsi;
  out[1] = t / (1.0 + R.rigid_over_2vs * dvdtau);
  out[2] = dsig;
}

__device__ __forceinline__ double slip_rate(double vref, double psi, double tau, double sig, double a) {
  return 2 * vref * exp(-psi / a) * sinh(tau / sig / a);
}

}  // namespace hbi
