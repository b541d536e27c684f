// hbi_matvec.cu -- phase 3 of the lattice H-matrix-vector product and the
// fused rate-and-state / Cash-Karp stage epilogue.
//
// Replaces HACApK_adot_lattice_hyp + HACApK_adot_body_lfmtx_hyp_contiguous
// (m_HACApK_solve.f90:220-337, 2108-2164) together with hbi_stream.cu, which
// holds phases 1 (z = V^T x) and 2 (partial row sums of U z + A x per row
// group and column chunk).  Phase 3 sums, per row, the partials of the row
// groups covering the row (coarse to fine, chunks in order) -- plain, or fused
// with the rate-and-state / RK stage epilogue (derivs/deriv/rkck,
// main_LH.f90:2053-2244, 2472-2554).  Every sum has a fixed order, so the
// product is deterministic without atomics.
#include <cuda_bf16.h>

#include "hbi_kernels.cuh"
#include "hbi_rsf.cuh"

namespace hbi {

__constant__ double cB[15];   // B21 B31 B32 B41 B42 B43 B51..B54 B61..B65
__constant__ double cC[6];    // C1 0 C3 C4 0 C6
__constant__ double cDC[6];   // DC1 0 DC3 DC4 DC5 DC6

void set_tableau(const double* B, const double* C, const double* DC) {
  cudaMemcpyToSymbol(cB, B, sizeof(double) * 15);
  cudaMemcpyToSymbol(cC, C, sizeof(double) * 6);
  cudaMemcpyToSymbol(cDC, DC, sizeof(double) * 6);
}

// phase 3: y(r) = scale * sum over the groups covering row r, coarse to
// fine.  The partials' offsets come from one flat list per fine range, so the
// loads of a row are independent of one another (three levels of latency
// whatever the tree depth); eight of them in flight at a time.
template <typename Acc>
__device__ __forceinline__ double group_sum(const MatDev& m, int r) {
  const Acc* gp = (const Acc*)m.gpart;
  const int f = __ldg(&m.row_fc[r]);
  const int e0 = __ldg(&m.fcb_ptr[f]), e1 = __ldg(&m.fcb_ptr[f + 1]);
  Acc s = 0;
  int e = e0;
  for (; e + 8 <= e1; e += 8) {
    Acc v[8];
#pragma unroll
    for (int u = 0; u < 8; u++) v[u] = __ldcg(gp + __ldg(&m.fcb_base[e + u]) + r);
#pragma unroll
    for (int u = 0; u < 8; u++) s += v[u];
  }
  for (; e < e1; e++) s += __ldcg(gp + __ldg(&m.fcb_base[e]) + r);
  return (double)s * m.scale;
}

__device__ __forceinline__ double row_value(const MatDev& m, int r) {
  return m.storage == ST_F64 ? group_sum<double>(m, r) : group_sum<float>(m, r);
}

__global__ void __launch_bounds__(256) p3_plain_kernel(MatDev m0, MatDev m1, int nmat, double* y0, double* y1) {
  pdl_launch_dependents();
  pdl_wait_prior();
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= m0.n) return;
  y0[r] = row_value(m0, r);
  if (nmat == 2) y1[r] = row_value(m1, r);
}

__global__ void __launch_bounds__(128) p3_rk_kernel(MatDev m0, MatDev m1, RkDev R, int s, double* __restrict__ xnext) {
  pdl_launch_dependents();
  pdl_wait_prior();
  if (R.flags && __ldcg(&R.flags[0])) return;
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  double emax = -1.0;
  long long hidx = -1;
  if (r < R.n) {
    const int n3 = 3 * R.n;
    double k[3];
    double* Ks = R.K + (size_t)s * n3 + 3 * r;
    if (s == 0 && R.flags && __ldcg(&R.flags[2])) {
      // a retried attempt from the same state: k1 = f(y) is the one the
      // rejected attempt stored (its phases 1-2 were skipped)
      k[0] = Ks[0]; k[1] = Ks[1]; k[2] = Ks[2];
    } else {
      const double gs = row_value(m0, r) + R.taudot[r];
      const double gn = (R.nmat == 2 ? row_value(m1, r) : 0.0) + R.sigdot[r];
      const double psi = R.ys[3 * r], tau = R.ys[3 * r + 1], sig = R.ys[3 * r + 2];
      deriv_dev(R, gs, gn, psi, tau, sig, R.vs[r], R.ws[r], R.a[r], R.b[r], R.dc[r], R.f0[r], k);
      Ks[0] = k[0]; Ks[1] = k[1]; Ks[2] = k[2];
    }
    const double h = R.ctl[0];
    const double* K0 = R.K + 3 * r;
    if (s < 5) {
      double yn[3];
#pragma unroll
      for (int c = 0; c < 3; c++) {
        const double y = R.y[3 * r + c];
        const double k1 = K0[c];
        double v;
        if (s == 0) {
          v = y + cB[0] * h * k[c];
        } else if (s == 1) {
          v = y + h * (cB[1] * k1 + cB[2] * k[c]);
        } else if (s == 2) {
          const double k2 = K0[n3 + c];
          v = y + h * (cB[3] * k1 + cB[4] * k2 + cB[5] * k[c]);
        } else if (s == 3) {
          const double k2 = K0[n3 + c], k3 = K0[2 * n3 + c];
          v = y + h * (cB[6] * k1 + cB[7] * k2 + cB[8] * k3 + cB[9] * k[c]);
        } else {
          const double k2 = K0[n3 + c], k3 = K0[2 * n3 + c], k4 = K0[3 * n3 + c];
          v = y + h * (cB[10] * k1 + cB[11] * k2 + cB[12] * k3 + cB[13] * k4 + cB[14] * k[c]);
        }
        yn[c] = v;
      }
      R.ys[3 * r] = yn[0]; R.ys[3 * r + 1] = yn[1]; R.ys[3 * r + 2] = yn[2];
      double vn, wn;
      slip_rate_w(R.vref, yn[0], yn[1], yn[2], R.a[r], &vn, &wn);
      R.vs[r] = vn;
      R.ws[r] = wn;
      xnext[r] = R.backslip ? (vn + 0.0) - R.vpl[r] : vn + 0.0;
    } else {
      const double eps = R.ctl[1];
#pragma unroll
      for (int c = 0; c < 3; c++) {
        const double y = R.y[3 * r + c];
        const double k1 = K0[c], k3 = K0[2 * n3 + c], k4 = K0[3 * n3 + c], k5 = K0[4 * n3 + c], k6 = k[c];
        const double yo = y + h * (cC[0] * k1 + cC[2] * k3 + cC[3] * k4 + cC[5] * k6);
        const double ye = h * (cDC[0] * k1 + cDC[2] * k3 + cDC[3] * k4 + cDC[4] * k5 + cDC[5] * k6);
        R.yout[3 * r + c] = yo;
        R.yerr[3 * r + c] = ye;
        const double e = fabs(ye / yo) / eps;
        R.ebuf[3 * r + c] = e;
        if (e > emax) emax = e;
        if (yo - 1 == yo) hidx = 3 * r + c;
      }
    }
  }
  if (s == 5) {
    // block-wide max of e (NaN never wins) and of the last huge index
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double oe = __shfl_xor_sync(0xffffffffu, emax, o);
      if (oe > emax) emax = oe;
      const long long oh = __shfl_xor_sync(0xffffffffu, hidx, o);
      if (oh > hidx) hidx = oh;
    }
    if ((threadIdx.x & 31) == 0) {
      if (emax >= 0.0) atomicMax((unsigned long long*)&R.ctl[2], (unsigned long long)__double_as_longlong(emax));
      if (hidx >= 0) atomicMax((long long*)&R.ctl[3], hidx);
    }
  }
}

// start of an attempt: stage state = accepted state, its slip rate and the
// stage-0 matvec input; clear the attempt's error accumulators
__global__ void rk_prepare_kernel(RkDev R) {
  pdl_launch_dependents();
  pdl_wait_prior();
  if (R.flags && __ldcg(&R.flags[0])) return;
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r == 0) {
    R.ctl[2] = 0.0;
    ((long long*)R.ctl)[3] = -1;
  }
  if (r >= R.n) return;
  const double psi = R.y[3 * r], tau = R.y[3 * r + 1], sig = R.y[3 * r + 2];
  R.ys[3 * r] = psi; R.ys[3 * r + 1] = tau; R.ys[3 * r + 2] = sig;
  double v, w;
  slip_rate_w(R.vref, psi, tau, sig, R.a[r], &v, &w);
  R.vs[r] = v;
  R.ws[r] = w;
  R.x0[r] = R.backslip ? (v + 0.0) - R.vpl[r] : v + 0.0;
}

// ------------------------------------------------------------- launchers
void launch_phase3_plain(const MatDev* mats, int nmat, double* const* y, cudaStream_t st) {
  const MatDev& m1 = nmat == 2 ? mats[1] : mats[0];
  launch_kernel(p3_plain_kernel, dim3((mats[0].n + 255) / 256), dim3(256), 0, st, pdl_enabled(), mats[0], m1, nmat,
                y[0], nmat == 2 ? y[1] : nullptr);
}

void launch_phase3_rk(const MatDev* mats, int nmat, const RkDev& rk, int stage, double* xnext, cudaStream_t st) {
  const MatDev& m1 = nmat == 2 ? mats[1] : mats[0];
  launch_kernel(p3_rk_kernel, dim3((rk.n + 127) / 128), dim3(128), 0, st, pdl_enabled(), mats[0], m1, rk, stage,
                xnext);
}

void launch_rk_prepare(const RkDev& rk, cudaStream_t st) {
  rk_prepare_kernel<<<(rk.n + 255) / 256, 256, 0, st>>>(rk);
}

}  // namespace hbi
