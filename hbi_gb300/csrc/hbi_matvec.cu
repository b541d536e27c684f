// hbi_matvec.cu -- lattice H-matrix-vector product and the fused
// rate-and-state / Cash-Karp stage epilogue.
//
// Replaces HACApK_adot_lattice_hyp + HACApK_adot_body_lfmtx_hyp_contiguous
// (m_HACApK_solve.f90:220-337, 2108-2164).  Three kernels per product:
//   phase 1  z_l = V_l^T x for every low-rank leaf (one warp per leaf row
//            chunk; leaves split over several chunks are summed by the
//            last-arriving warp in a fixed order);
//   phase 2  per row group (the leaves sharing one row range) and chunk of
//            rows: sum of U_l z_l and A_l x over the group's leaves;
//   phase 3  per row: sum of the partials of the groups covering the row,
//            coarse to fine -- plain, or fused with the rate-and-state / RK
//            stage epilogue (derivs/deriv/rkck, main_LH.f90:2053-2244,
//            2472-2554).
// Every sum has a fixed order, so the product is deterministic without atomics.
// Factors are column-major (V: ndt x kt, U: ndl x kt, dense A: ndl x ndt), each
// column zero-padded to 16 bytes, in FP64, FP32 or BF16; FP32/BF16 storage
// accumulates in FP32.  All factor reads are 16-byte vector loads.
#include <cuda_bf16.h>

#include <map>
#include <mutex>

#include "hbi_kernels.cuh"

namespace hbi {

__constant__ double cB[15];   // B21 B31 B32 B41 B42 B43 B51..B54 B61..B65
__constant__ double cC[6];    // C1 0 C3 C4 0 C6
__constant__ double cDC[6];   // DC1 0 DC3 DC4 DC5 DC6

void set_tableau(const double* B, const double* C, const double* DC) {
  cudaMemcpyToSymbol(cB, B, sizeof(double) * 15);
  cudaMemcpyToSymbol(cC, C, sizeof(double) * 6);
  cudaMemcpyToSymbol(cDC, DC, sizeof(double) * 6);
}

template <typename T> struct AccOf { typedef float type; };
template <> struct AccOf<double> { typedef double type; };

__device__ __forceinline__ double ld_acc(const double* p) { return __ldg(p); }
__device__ __forceinline__ float ld_acc(const float* p) { return __ldg(p); }
__device__ __forceinline__ float ld_acc(const __nv_bfloat16* p) { return __bfloat162float(__ldg(p)); }

// ---------------------------------------------------------------- vectors
// 16-byte loads: 4 floats, 2 doubles or 8 bf16 (widened to float)
__device__ __forceinline__ void ldv(const float* p, float* o) {
  const float4 v = __ldg(reinterpret_cast<const float4*>(p));
  o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
}
__device__ __forceinline__ void ldv(const double* p, double* o) {
  const double2 v = __ldg(reinterpret_cast<const double2*>(p));
  o[0] = v.x; o[1] = v.y;
}
__device__ __forceinline__ void ldv(const __nv_bfloat16* p, float* o) {
  const uint4 v = __ldg(reinterpret_cast<const uint4*>(p));
  const unsigned w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
  for (int i = 0; i < 4; i++) {
    o[2 * i] = __uint_as_float(w[i] << 16);
    o[2 * i + 1] = __uint_as_float(w[i] & 0xffff0000u);
  }
}
// smallest power of two >= n, as a shift (n in 1..32)
__device__ __forceinline__ int log2ceil32(int n) { return n <= 1 ? 0 : 32 - __clz(n - 1); }

// ---------------------------------------------------------------- phase 1
// z_l = V_l^T x.  V is column-major, each column padded to a multiple of VEC
// rows.  A warp task covers rows [t0, t0+nt) of every column of one leaf.
// The lanes form CS = 32/LW column slots of LW lanes; lane j of a slot reads
// rows [j*VEC, j*VEC+VEC) of its column with one 16-byte load, so a warp
// instruction moves CS column segments at once and four such columns are in
// flight per lane.  Each column's sum is reduced over the LW lanes of its slot.
template <typename T>
__global__ void __launch_bounds__(256) p1_kernel(MatDev m0, MatDev m1, int nmat, const double* __restrict__ x) {
  typedef typename AccOf<T>::type Acc;
  constexpr int VEC = 16 / sizeof(T);
  if (m0.skip && __ldcg(m0.skip)) return;
  const int lane = threadIdx.x & 31;
  const int warp = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
  const int nwarps = (int)((gridDim.x * (int64_t)blockDim.x) >> 5);
  // the tasks of both H-matrices (shear, normal) in one grid: m0's, then m1's
  const int n0 = m0.np1, ntot = nmat == 2 ? n0 + m1.np1 : n0;
  for (int it = warp; it < ntot; it += nwarps) {
    const bool sec = it >= n0;
    const T* store = (const T*)(sec ? m1.store : m0.store);
    Acc* part = (Acc*)(sec ? m1.part : m0.part);
    Acc* z = (Acc*)(sec ? m1.z : m0.z);
    const LrInfo* lrt = sec ? m1.lr : m0.lr;
    int* cnt = sec ? m1.lr_cnt : m0.lr_cnt;
    const P1ItemDev I = (sec ? m1.p1 : m0.p1)[sec ? it - n0 : it];
    const int nq = (I.nt + VEC - 1) / VEC;
    const int lw = log2ceil32(min(nq, 32));
    const int LW = 1 << lw, CS = 32 >> lw;
    const int slot = lane >> lw, j = lane & (LW - 1);
    const T* V = store + I.voff;
    const int64_t ld = I.ldv;
    const LrInfo L = lrt[I.lr];
    Acc* dst = L.nparts == 1 ? z : part;
    for (int kb = 0; kb < I.nk; kb += 4 * CS) {
      Acc s[4] = {0, 0, 0, 0};
      for (int q = j; q < nq; q += LW) {
        const int t = q * VEC;
        Acc xv[VEC], a[4][VEC];
        // all loads of the step first; columns past nk re-read column 0 and
        // are dropped at the write
#pragma unroll
        for (int u = 0; u < 4; u++) {
          const int k = kb + u * CS + slot;
          ldv(V + (k < I.nk ? k : 0) * ld + t, a[u]);
        }
#pragma unroll
        for (int v = 0; v < VEC; v++) xv[v] = (t + v < I.nt) ? (Acc)__ldg(&x[I.x0 + t + v]) : Acc(0);
#pragma unroll
        for (int u = 0; u < 4; u++)
#pragma unroll
          for (int v = 0; v < VEC; v++) s[u] += a[u][v] * xv[v];
      }
#pragma unroll
      for (int u = 0; u < 4; u++)
        for (int o = 1; o < LW; o <<= 1) s[u] += __shfl_xor_sync(0xffffffffu, s[u], o);
      if (j == 0) {
#pragma unroll
        for (int u = 0; u < 4; u++) {
          const int k = kb + u * CS + slot;
          if (k < I.nk) dst[I.pout + k] = s[u];
        }
      }
    }
    if (L.nparts > 1) {
      __threadfence();
      int last = 0;
      if (lane == 0) last = (atomicAdd(&cnt[I.lr], 1) == L.nitems - 1);
      last = __shfl_sync(0xffffffffu, last, 0);
      if (last) {
        __threadfence();
        for (int k = lane; k < L.kt; k += 32) {
          Acc s = 0;
          for (int p = 0; p < L.nparts; p++) s += __ldcg(&part[L.poff + p * L.kt + k]);
          z[L.zoff + k] = s;
        }
        if (lane == 0) cnt[I.lr] = 0;
      }
    }
  }
}

// ---------------------------------------------------------------- phase 2
// One warp per (row group, chunk of up to 32*VEC rows).  Lane j of column
// slot `slot` owns rows [j*VEC, j*VEC+VEC) of the chunk; slots take different
// columns (k) of the same leaf, and the group's leaves are walked in order
// with their descriptors fetched 32 at a time and broadcast by shuffles.  The
// slots' partial row sums are combined at the end.  All lanes run the same
// loop trip counts, so the shuffles are convergent.
template <typename T>
__global__ void __launch_bounds__(256, 3) p2_group_kernel(MatDev m0, MatDev m1, int nmat,
                                                          const double* __restrict__ x) {
  typedef typename AccOf<T>::type Acc;
  constexpr int VEC = 16 / sizeof(T);
  constexpr int UNR = VEC >= 8 ? 2 : 4;
  if (m0.skip && __ldcg(m0.skip)) return;
  const int lane = threadIdx.x & 31;
  const int warp = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
  const int nwarps = (int)((gridDim.x * (int64_t)blockDim.x) >> 5);
  const int n0 = m0.np2, ntot = nmat == 2 ? n0 + m1.np2 : n0;
  for (int it = warp; it < ntot; it += nwarps) {
    const bool sec = it >= n0;
    const int32_t* gleaf_ptr = sec ? m1.gleaf_ptr : m0.gleaf_ptr;
    const int32_t* gleaf = sec ? m1.gleaf : m0.gleaf;
    const LeafDescDev* desc = sec ? m1.desc : m0.desc;
    const int32_t* gpoff = sec ? m1.gpoff : m0.gpoff;
    const T* store = (const T*)(sec ? m1.store : m0.store);
    const Acc* z = (const Acc*)(sec ? m1.z : m0.z);
    Acc* gpart = (Acc*)(sec ? m1.gpart : m0.gpart);
    const P2ItemDev I = (sec ? m1.p2 : m0.p2)[sec ? it - n0 : it];
    const int g = I.group;
    const int nq = (I.nr + VEC - 1) / VEC;
    const int lw = log2ceil32(min(nq, 32));
    const int LW = 1 << lw, CS = 32 >> lw;
    const int slot = lane >> lw, j = lane & (LW - 1);
    const bool act = j < nq;
    const int rr = I.r0 + j * VEC;
    Acc acc[VEC];
#pragma unroll
    for (int v = 0; v < VEC; v++) acc[v] = 0;
    const int e0 = __ldg(&gleaf_ptr[g]), e1 = __ldg(&gleaf_ptr[g + 1]);
    for (int base = e0; base < e1; base += 32) {
      const int nl = min(32, e1 - base);
      long long my_off = 0;
      int my_ld = 0, my_kind = 0, my_cnt = 0, my_aux = 0;
      if (lane < nl) {
        const LeafDescDev* d = desc + __ldg(&gleaf[base + lane]);
        my_off = __ldg(&d->off);
        my_ld = __ldg(&d->ndl);
        my_kind = __ldg(&d->kind);
        my_cnt = __ldg(&d->kt_or_ndt);
        my_aux = __ldg(&d->aux);
      }
      for (int jl = 0; jl < nl; jl++) {
        const long long off = __shfl_sync(0xffffffffu, my_off, jl);
        const int64_t ld = __shfl_sync(0xffffffffu, my_ld, jl);
        const int kind = __shfl_sync(0xffffffffu, my_kind, jl);
        const int cnt = __shfl_sync(0xffffffffu, my_cnt, jl);
        const int aux = __shfl_sync(0xffffffffu, my_aux, jl);
        const T* P = store + off + (act ? rr : 0);
        for (int kb = 0; kb < cnt; kb += UNR * CS) {
          // issue every load of the unrolled step before the first FMA;
          // out-of-range columns read column 0 and are multiplied by zero
          Acc a[UNR][VEC], mu[UNR];
#pragma unroll
          for (int u = 0; u < UNR; u++) {
            const int k = kb + u * CS + slot;
            const bool ok = act && k < cnt;
            const int kk = ok ? k : 0;
            ldv(P + kk * ld, a[u]);
            if (kind == 1) mu[u] = ok ? z[aux + kk] : Acc(0);
            else mu[u] = ok ? (Acc)__ldg(&x[aux + kk]) : Acc(0);
          }
#pragma unroll
          for (int u = 0; u < UNR; u++)
#pragma unroll
            for (int v = 0; v < VEC; v++) acc[v] += a[u][v] * mu[u];
        }
      }
    }
#pragma unroll
    for (int v = 0; v < VEC; v++)
      for (int o = LW; o < 32; o <<= 1) acc[v] += __shfl_xor_sync(0xffffffffu, acc[v], o);
    if (slot == 0 && act) {
      const int gp = __ldg(&gpoff[g]);
#pragma unroll
      for (int v = 0; v < VEC; v++)
        if (rr + v < I.r0 + I.nr) gpart[gp + rr + v] = acc[v];
    }
  }
}

// phase 3: y(r) = scale * sum over the groups covering row r, coarse to fine
template <typename Acc>
__device__ __forceinline__ double group_sum(const MatDev& m, int r) {
  const Acc* gp = (const Acc*)m.gpart;
  const int f = __ldg(&m.row_fc[r]);
  const int e0 = __ldg(&m.fc_ptr[f]), e1 = __ldg(&m.fc_ptr[f + 1]);
  Acc s = 0;
  for (int e = e0; e < e1; e++) {
    const int g = __ldg(&m.fc_group[e]);
    s += __ldcg(&gp[__ldg(&m.gpoff[g]) + r - __ldg(&m.grow0[g])]);
  }
  return (double)s * m.scale;
}

__device__ __forceinline__ double row_value(const MatDev& m, int r) {
  return m.storage == ST_F64 ? group_sum<double>(m, r) : group_sum<float>(m, r);
}

__global__ void __launch_bounds__(256) p3_plain_kernel(MatDev m0, MatDev m1, int nmat, double* y0, double* y1) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= m0.n) return;
  y0[r] = row_value(m0, r);
  if (nmat == 2) y1[r] = row_value(m1, r);
}

// deriv (main_LH.f90:2165-2244): aging (0) and slip (1) laws
__device__ __forceinline__ void deriv_dev(const RkDev& R, double sum_gs, double sum_gn, double psi, double tau,
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

__global__ void __launch_bounds__(128) p3_rk_kernel(MatDev m0, MatDev m1, RkDev R, int s, double* __restrict__ xnext) {
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
      deriv_dev(R, gs, gn, psi, tau, sig, R.vs[r], R.a[r], R.b[r], R.dc[r], R.f0[r], k);
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
      const double vn = slip_rate(R.vref, yn[0], yn[1], yn[2], R.a[r]);
      R.vs[r] = vn;
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
  if (R.flags && __ldcg(&R.flags[0])) return;
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r == 0) {
    R.ctl[2] = 0.0;
    ((long long*)R.ctl)[3] = -1;
  }
  if (r >= R.n) return;
  const double psi = R.y[3 * r], tau = R.y[3 * r + 1], sig = R.y[3 * r + 2];
  R.ys[3 * r] = psi; R.ys[3 * r + 1] = tau; R.ys[3 * r + 2] = sig;
  const double v = slip_rate(R.vref, psi, tau, sig, R.a[r]);
  R.vs[r] = v;
  R.x0[r] = R.backslip ? (v + 0.0) - R.vpl[r] : v + 0.0;
}

// FP64 HACApK body -> matvec store (type T): low rank [V][U] unchanged,
// dense a1(ndt,ndl) transposed to column-major ndl x ndt
template <typename T>
__device__ __forceinline__ T cvt(double v);
template <> __device__ __forceinline__ double cvt<double>(double v) { return v; }
template <> __device__ __forceinline__ float cvt<float>(double v) { return (float)v; }
template <> __device__ __forceinline__ __nv_bfloat16 cvt<__nv_bfloat16>(double v) { return __double2bfloat16(v); }

template <typename T>
__global__ void store_convert_kernel(const double* __restrict__ src, int nleaf, const int64_t* src_off,
                                     const int64_t* dst_off, const int32_t* kind, const int32_t* rows,
                                     const int32_t* cols, const int32_t* kts, T* dst) {
  // columns padded to multiples of VEC rows (16 bytes); the store is zeroed
  // beforehand, so pad rows stay zero
  constexpr int VEC = 16 / sizeof(T);
  for (int lf = blockIdx.x; lf < nleaf; lf += gridDim.x) {
    const double* s = src + src_off[lf];
    T* d = dst + dst_off[lf];
    const int ndl = rows[lf], ndt = cols[lf];
    const int64_t ndlp = (ndl + VEC - 1) / VEC * VEC;
    if (kind[lf] == 1) {
      // [V: ndtp x kt][U: ndlp x kt], column-major, from [V: ndt x kt][U: ndl x kt]
      const int kt = kts[lf];
      const int64_t ndtp = (ndt + VEC - 1) / VEC * VEC;
      const int64_t nv = (int64_t)kt * ndt, nu = (int64_t)kt * ndl;
      for (int64_t e = threadIdx.x; e < nv; e += blockDim.x) {
        const int64_t k = e / ndt, t = e % ndt;
        d[k * ndtp + t] = cvt<T>(s[e]);
      }
      T* du = d + ndtp * kt;
      for (int64_t e = threadIdx.x; e < nu; e += blockDim.x) {
        const int64_t k = e / ndl, i = e % ndl;
        du[k * ndlp + i] = cvt<T>(s[nv + e]);
      }
    } else {
      // A(il, it) column-major with leading dimension ndlp, from a1(ndt, ndl)
      const int64_t ne = (int64_t)ndl * ndt;
      for (int64_t e = threadIdx.x; e < ne; e += blockDim.x) {
        const int64_t it = e / ndl, il = e % ndl;
        d[it * ndlp + il] = cvt<T>(s[il * ndt + it]);
      }
    }
  }
}

// ------------------------------------------------------------- launchers
// persistent grid: as many 256-thread blocks as are resident at once (one
// wave), never more than the items need
template <typename K>
static int grid_for(K kernel, int sm, int nitems) {
  // resident blocks per SM, cached per kernel (function address)
  static std::mutex mu;
  static std::map<const void*, int> cache;
  int per_sm;
  {
    std::lock_guard<std::mutex> lock(mu);
    auto it = cache.find((const void*)kernel);
    if (it == cache.end()) {
      int nb = 0;
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, 256, 0) != cudaSuccess || nb < 1) nb = 2;
      it = cache.emplace((const void*)kernel, nb).first;
    }
    per_sm = it->second;
  }
  const int full = per_sm * sm;
  const int need = (nitems + 7) / 8;
  return need < full ? (need > 0 ? need : 1) : full;
}

// both H-matrices of a stage in one grid per phase (same storage type)
void launch_phase1(const MatDev* mats, int nmat, const double* x, int sm, cudaStream_t st) {
  const MatDev& m0 = mats[0];
  const MatDev& m1 = nmat == 2 ? mats[1] : mats[0];
  const int n = m0.np1 + (nmat == 2 ? m1.np1 : 0);
  if (n == 0) return;
  if (m0.storage == ST_F64)
    p1_kernel<double><<<grid_for(p1_kernel<double>, sm, n), 256, 0, st>>>(m0, m1, nmat, x);
  else if (m0.storage == ST_F32)
    p1_kernel<float><<<grid_for(p1_kernel<float>, sm, n), 256, 0, st>>>(m0, m1, nmat, x);
  else
    p1_kernel<__nv_bfloat16><<<grid_for(p1_kernel<__nv_bfloat16>, sm, n), 256, 0, st>>>(m0, m1, nmat, x);
}

void launch_phase2(const MatDev* mats, int nmat, const double* x, int sm, cudaStream_t st) {
  const MatDev& m0 = mats[0];
  const MatDev& m1 = nmat == 2 ? mats[1] : mats[0];
  const int n = m0.np2 + (nmat == 2 ? m1.np2 : 0);
  if (n == 0) return;
  if (m0.storage == ST_F64)
    p2_group_kernel<double><<<grid_for(p2_group_kernel<double>, sm, n), 256, 0, st>>>(m0, m1, nmat, x);
  else if (m0.storage == ST_F32)
    p2_group_kernel<float><<<grid_for(p2_group_kernel<float>, sm, n), 256, 0, st>>>(m0, m1, nmat, x);
  else
    p2_group_kernel<__nv_bfloat16><<<grid_for(p2_group_kernel<__nv_bfloat16>, sm, n), 256, 0, st>>>(m0, m1, nmat, x);
}

void launch_phase3_plain(const MatDev* mats, int nmat, double* const* y, cudaStream_t st) {
  const MatDev& m1 = nmat == 2 ? mats[1] : mats[0];
  p3_plain_kernel<<<(mats[0].n + 255) / 256, 256, 0, st>>>(mats[0], m1, nmat, y[0], nmat == 2 ? y[1] : nullptr);
}

void launch_phase3_rk(const MatDev* mats, int nmat, const RkDev& rk, int stage, double* xnext, cudaStream_t st) {
  const MatDev& m1 = nmat == 2 ? mats[1] : mats[0];
  p3_rk_kernel<<<(rk.n + 127) / 128, 128, 0, st>>>(mats[0], m1, rk, stage, xnext);
}

void launch_rk_prepare(const RkDev& rk, cudaStream_t st) {
  rk_prepare_kernel<<<(rk.n + 255) / 256, 256, 0, st>>>(rk);
}

void launch_store_convert(const double* src, const LeafDescDev*, int nleaf, const int64_t* src_off,
                          const int64_t* dst_off, const int32_t* kind, const int32_t* rows, const int32_t* cols,
                          const int32_t* kts, void* dst, int storage, cudaStream_t st) {
  int blocks = nleaf < 152 * 16 ? (nleaf > 0 ? nleaf : 1) : 152 * 16;
  if (storage == ST_F64)
    store_convert_kernel<double><<<blocks, 256, 0, st>>>(src, nleaf, src_off, dst_off, kind, rows, cols, kts, (double*)dst);
  else if (storage == ST_F32)
    store_convert_kernel<float><<<blocks, 256, 0, st>>>(src, nleaf, src_off, dst_off, kind, rows, cols, kts, (float*)dst);
  else
    store_convert_kernel<__nv_bfloat16><<<blocks, 256, 0, st>>>(src, nleaf, src_off, dst_off, kind, rows, cols, kts,
                                                                (__nv_bfloat16*)dst);
}

}  // namespace hbi
