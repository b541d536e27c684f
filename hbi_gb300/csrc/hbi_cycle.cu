// hbi_cycle.cu -- the earthquake-cycle time loop on the device.
//
// The reference's loop (main_LH.f90:1217-1438) calls rkqs, updates slip and
// slip rate (:1266-1287), reduces the monitors (:1291-1336), detects events
// (:1338-1388), writes fields (:1391-1412) and applies the stop controls
// (:1425-1438), all on the host with a synchronisation per step.  Here one
// CUDA graph per RK attempt carries the whole decision chain:
//
//   rk_prepare, 6 x (phase 1, phase 2, phase 3 + RK epilogue)   the attempt
//   cycle_control   errmax, accept/reject, next h (rkqs :2296-2360); stops
//                   the loop if a product kernel gave up a bulk-copy wait
//   cycle_update    y <- ytemp, slip, slip rate, monitors, event state,
//                   output decision, stop controls
//   cycle_snapshot  fields into a ring slot when the step writes output
//   cycle_record    the loop state into a host-mapped record ring
//
// so the host never decides anything before the next attempt can start: it
// keeps `inflight` attempts enqueued and drains their records into the
// reference's output files.  A halted loop (stop control, step or time limit)
// turns the attempts already enqueued into no-ops.  A retried attempt (after a
// rejection) re-uses the stage-1 derivative of the rejected one: f(y) does not
// depend on h, so phases 1-2 of stage 1 are skipped.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstddef>
#include <cstring>
#include <deque>
#include <string>
#include <vector>

#include "../../include/hbi_gpu.h"
#include "hbi_kernels.cuh"
#include "hbi_rsf.cuh"

namespace hbi {
int rk_view(hbi_rk* r, RkView* v);
int set_error(int code, const char* msg);

namespace {

// run constants of a loop
struct CycleConst {
  int n, nsnap, nrec, pad;
  double eps, dtmax, tmax, velth, velmax, velmin, dtout_inter, dtout_co, sg;
  long long interval;
};

// the loop state; lives on the device, one copy per attempt goes to the host
struct CycleState {
  double x, h, h_try, hdid, hnext, errmax, h_pending;
  double mvel, meanslip, meanmu, maxnorm, minnorm;
  double tout, dtout, moment0, moment, onset, t_limit;
  double hist_e1, hist_h1, hist_v1, hist_v2;  // history for the learned proposer
  double proposal;                             // log(h_next / rkqs h_next) of the proposer
  long long k, attempt, launch, k_limit, rejected;
  int nrjct, nr, accepted, halted, stop, slipping, eventcount, hypoloc;
  int loc, outfield, ev, snap, nsnap_used, clamped, skipped, learned;
  unsigned int arrive, pad;
};

// learned step-size proposer: weights of the MLP (float), standardisation of
// its inputs and the clamp of its output (hbi_mlp.cu trains it).  Layout:
// W1[hid][nin] b1[hid] W2[hid][hid] b2[hid] W3[hid] b3 mean[nin] sd[nin] lo hi
struct ProposerDev {
  const float* w;
  int nin, hid;
};

struct MonPart {
  double vmax;
  long long imax;
  double smax, smin, sslip, smu;
};

__device__ __forceinline__ MonPart mon_identity() {
  MonPart m;
  m.vmax = -1.0;
  m.imax = 0x7fffffffffffffffLL;
  m.smax = -INFINITY;
  m.smin = INFINITY;
  m.sslip = 0.0;
  m.smu = 0.0;
  return m;
}

// maxloc keeps the first index of the largest |v| (Fortran maxloc)
__device__ __forceinline__ void mon_combine(MonPart& a, const MonPart& b) {
  if (b.vmax > a.vmax || (b.vmax == a.vmax && b.imax < a.imax)) {
    a.vmax = b.vmax;
    a.imax = b.imax;
  }
  a.smax = fmax(a.smax, b.smax);
  a.smin = fmin(a.smin, b.smin);
  a.sslip += b.sslip;
  a.smu += b.smu;
}

// fixed-order block reduction (256 threads): butterfly in each warp, warps in order
__device__ MonPart mon_block_reduce(MonPart m, MonPart* sh) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    MonPart b;
    b.vmax = __shfl_xor_sync(0xffffffffu, m.vmax, o);
    b.imax = __shfl_xor_sync(0xffffffffu, m.imax, o);
    b.smax = __shfl_xor_sync(0xffffffffu, m.smax, o);
    b.smin = __shfl_xor_sync(0xffffffffu, m.smin, o);
    b.sslip = __shfl_xor_sync(0xffffffffu, m.sslip, o);
    b.smu = __shfl_xor_sync(0xffffffffu, m.smu, o);
    // combine in lane order so both partners hold the same sums
    if ((threadIdx.x & o) == 0) {
      mon_combine(m, b);
    } else {
      mon_combine(b, m);
      m = b;
    }
  }
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = m;
  __syncthreads();
  MonPart r = sh[0];
  for (int w = 1; w < (int)(blockDim.x >> 5); w++) mon_combine(r, sh[w]);
  return r;
}

// rkqs constants (main_LH.f90:2290): default-real literals widened to real(8)
#define RK_SAFETY ((double)0.9f)
#define RK_PGROW ((double)-0.2f)
#define RK_PSHRNK (-0.25)
#define RK_TINY ((double)1e-20f)

__device__ double proposer_eval(const ProposerDev& M, const float* in, float* sh_a1, float* sh_a2) {
  // 3-layer MLP (tanh, tanh, linear) by the first `hid` threads of the block
  const float* W1 = M.w;
  const float* b1 = W1 + M.hid * M.nin;
  const float* W2 = b1 + M.hid;
  const float* b2 = W2 + M.hid * M.hid;
  const float* W3 = b2 + M.hid;
  const float* b3 = W3 + M.hid;
  const int o = threadIdx.x;
  if (o < M.hid) {
    float z = b1[o];
    for (int i = 0; i < M.nin; i++) z += W1[o * M.nin + i] * in[i];
    sh_a1[o] = tanhf(z);
  }
  __syncthreads();
  if (o < M.hid) {
    float z = b2[o];
    for (int i = 0; i < M.hid; i++) z += W2[o * M.hid + i] * sh_a1[i];
    sh_a2[o] = tanhf(z);
  }
  __syncthreads();
  float y = b3[0];
  for (int i = 0; i < M.hid; i++) y += W3[i] * sh_a2[i];
  return (double)y;
}

}  // namespace

// the proposer network: inputs, hidden width; the feature order is shared
// with the trainer
#define HBI_PROPOSER_NIN 7
#define HBI_PROPOSER_HID 64
__host__ __device__ constexpr int proposer_weights(int nin, int hid) {
  return hid * nin + hid + hid * hid + hid + hid + 1;
}

// the proposer's features, all known once step k is accepted and before step
// k+1 is tried: this step's error and the previous one's, the step growth,
// the slip-rate trend of the last two steps, the rejections of this step, the
// rkqs growth factor and the maximum slip rate
__host__ __device__ inline void proposer_features(double e, double e_prev, double h, double h_prev, double v1,
                                                  double v2, int nrjct, double hnext, float* f) {
  const double tiny = 1e-30;
  f[0] = (float)log10(fmax(e, tiny));
  f[1] = (float)log10(fmax(e_prev, tiny));
  f[2] = (float)log10(fmax(h, tiny) / fmax(h_prev, tiny));
  f[3] = (float)(log10(fmax(v1, tiny)) - log10(fmax(v2, tiny)));
  f[4] = (float)nrjct;
  f[5] = (float)log10(fmax(hnext, tiny) / fmax(h, tiny));
  f[6] = (float)log10(fmax(v1, tiny));
}

namespace {

__global__ void __launch_bounds__(256) cycle_control_kernel(RkDev R, CycleConst P, CycleState* S, int* flags,
                                                            ProposerDev M, const int* err0, const int* err1) {
  __shared__ double red[8];
  __shared__ int halted;
  __shared__ float feat[16], a1[128], a2[128];
  __shared__ int use_mlp;
  if (threadIdx.x == 0) {
    halted = S->halted;
    // a product kernel of this attempt gave up a wait: its result is invalid,
    // the loop stops here (the attempt is recorded as not accepted)
    if (!halted && ((err0 && __ldcg(err0)) || (err1 && __ldcg(err1)))) {
      S->attempt += 1;
      S->accepted = 0;
      S->stop = HBI_STOP_DEVICE;
      S->halted = 1;
      flags[0] = 1;
      flags[1] = 1;
      halted = 2;
    }
  }
  __syncthreads();
  if (halted) {
    if (threadIdx.x == 0 && halted == 1) {
      S->accepted = 0;
      S->skipped = 1;
    }
    return;
  }
  double e = __ldcg(&R.ctl[2]);
  const long long hidx = __ldcg(&((const long long*)R.ctl)[3]);
  if (hidx >= 0) {
    // a component with ytemp-1 == ytemp resets errmax to 10; only later
    // components can raise it (main_LH.f90:2309-2313)
    double m = -1.0;
    for (long long c = hidx + 1 + threadIdx.x; c < 3LL * R.n; c += blockDim.x) {
      const double v = R.ebuf[c];
      if (v > m) m = v;
    }
    for (int o = 16; o > 0; o >>= 1) {
      const double t = __shfl_xor_sync(0xffffffffu, m, o);
      if (t > m) m = t;
    }
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    e = 10.0;
    for (int w = 0; w < 8; w++)
      if (red[w] > e) e = red[w];
  }
  double next = 0.0;
  if (threadIdx.x == 0) {
    const double h = R.ctl[0];
    S->h_try = h;
    S->errmax = e;
    S->attempt += 1;
    use_mlp = 0;
    if (e < 1.0 && e > RK_TINY) {
      double hn = fmin(2 * h, RK_SAFETY * h * pow(e, RK_PGROW));
      hn = fmin(hn, P.dtmax);
      S->hdid = h;
      S->hnext = hn;
      S->x = S->clamped ? S->t_limit : S->x + h;
      S->k += 1;
      S->nrjct = S->nr;
      S->nr = 0;
      S->accepted = 1;
      next = hn;
      if (S->clamped && S->h_pending > next) next = S->h_pending;
      S->clamped = 0;
      flags[2] = 0;
      if (S->learned && M.w) {
        // inputs of the proposer: this step against the history of the loop
        float f[HBI_PROPOSER_NIN];
        proposer_features(e, S->hist_e1, h, S->hist_h1, S->mvel, S->hist_v1, S->nrjct, hn, f);
        const float* mean = M.w + proposer_weights(M.nin, M.hid);
        const float* sd = mean + M.nin;
        for (int i = 0; i < M.nin; i++) feat[i] = (f[i] - mean[i]) / sd[i];
        use_mlp = 1;
      }
      S->hist_e1 = e;
      S->hist_h1 = h;
      S->hist_v2 = S->hist_v1;
      S->hist_v1 = S->mvel;
    } else {
      S->accepted = 0;
      S->nr += 1;
      S->rejected += 1;
      double hs = (e > RK_TINY) ? fmax(0.5 * h, RK_SAFETY * h * pow(e, RK_PSHRNK)) : 0.5 * h;
      const double xnew = S->x + hs;
      next = hs;
      flags[2] = 1;
      if (xnew - S->x < 1.e-15) {
        S->stop = HBI_STOP_UNDERFLOW;
        S->halted = 1;
        flags[0] = 1;
      }
    }
    red[0] = next;
  }
  __syncthreads();
  if (use_mlp) {
    // every thread takes part (the layers are split over threads)
    double d = proposer_eval(M, feat, a1, a2);
    if (threadIdx.x == 0) {
      if (!(d == d)) d = 0.0;
      const float* lohi = M.w + proposer_weights(M.nin, M.hid) + 2 * M.nin;
      d = fmin(fmax(d, (double)lohi[0]), (double)lohi[1]);
      // after a step that needed retries, never propose more than rkqs does
      if (S->nrjct > 0) d = fmin(d, 0.0);
      S->proposal = d;
      red[0] = fmin(red[0] * exp(d * 2.302585092994046), P.dtmax);
    }
  }
  if (threadIdx.x == 0) {
    next = red[0];
    // land exactly on the run's time limit
    if (S->x + next > S->t_limit) {
      S->h_pending = next;
      next = S->t_limit - S->x;
      S->clamped = 1;
    }
    if (S->accepted && S->x >= S->t_limit) {
      S->stop = HBI_STOP_TLIMIT;
      S->halted = 1;
      flags[0] = 1;
      next = S->h_pending;
      S->clamped = 0;
    }
    S->h = next;
    R.ctl[0] = next;
    flags[1] = flags[0] | flags[2];
  }
}

// accepted step: y <- ytemp; slip and slip rate (main_LH.f90:1266-1287); the
// monitors (:1291-1336) by a fixed-order two-level reduction; then, in the
// last block, the event state machine, output decision and stop controls
__global__ void __launch_bounds__(256) cycle_update_kernel(RkDev R, CycleConst P, CycleState* S, int* flags,
                                                           double* __restrict__ vel, double* __restrict__ slip,
                                                           const double* __restrict__ ds, MonPart* part, int init) {
  __shared__ MonPart sh[8];
  __shared__ int last;
  if (!init && !__ldcg(&S->accepted)) return;
  const double dt = init ? 0.0 : __ldcg(&S->hdid);
  MonPart m = mon_identity();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P.n; i += gridDim.x * blockDim.x) {
    double psi, tau, sig, v, s;
    if (init) {
      psi = R.y[3 * i];
      tau = R.y[3 * i + 1];
      sig = R.y[3 * i + 2];
      v = vel[i];
      s = slip[i];
    } else {
      psi = R.yout[3 * i];
      tau = R.yout[3 * i + 1];
      sig = R.yout[3 * i + 2];
      R.y[3 * i] = psi;
      R.y[3 * i + 1] = tau;
      R.y[3 * i + 2] = sig;
      s = slip[i] + (vel[i] + 0.0) * dt * 0.5;
      v = slip_rate(R.vref, psi, tau, sig, R.a[i]);
      s = s + (v + 0.0) * dt * 0.5;
      slip[i] = s;
      vel[i] = v;
    }
    const double mu = tau / sig;
    const double av = fabs(v);
    if (av > m.vmax) {
      m.vmax = av;
      m.imax = i;
    }
    m.smax = fmax(m.smax, sig);
    m.smin = fmin(m.smin, sig);
    m.sslip += (init ? s : fabs(s)) * ds[i];
    m.smu += mu * ds[i];
  }
  m = mon_block_reduce(m, sh);
  if (threadIdx.x == 0) {
    part[blockIdx.x] = m;
    __threadfence();
    last = atomicAdd(&S->arrive, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  MonPart f = mon_identity();
  for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) {
    MonPart q;
    q.vmax = __ldcg(&part[b].vmax);
    q.imax = __ldcg(&part[b].imax);
    q.smax = __ldcg(&part[b].smax);
    q.smin = __ldcg(&part[b].smin);
    q.sslip = __ldcg(&part[b].sslip);
    q.smu = __ldcg(&part[b].smu);
    mon_combine(f, q);
  }
  __syncthreads();
  f = mon_block_reduce(f, sh);
  if (threadIdx.x != 0) return;
  S->arrive = 0;
  S->mvel = f.vmax;
  S->loc = (int)f.imax;
  S->maxnorm = f.smax;
  S->minnorm = f.smin;
  S->meanslip = f.sslip / P.sg;
  S->meanmu = f.smu / P.sg;
  if (init) return;
  // event list (main_LH.f90:1338-1388)
  int outf = 0, ev = 0;
  if (!S->slipping && f.vmax > P.velth) {
    outf = 1;
    S->slipping = 1;
    S->dtout = P.dtout_co;
    S->tout = S->x + S->dtout;
    S->eventcount += 1;
    S->moment0 = S->meanslip;
    ev |= 1;
    S->hypoloc = (int)f.imax + 1;
    S->onset = S->x;
  }
  if (S->slipping && f.vmax < 0.5 * P.velth) {
    outf = 1;
    S->slipping = 0;
    S->dtout = P.dtout_inter;
    S->tout = S->x + S->dtout;
    S->moment = S->meanslip - S->moment0;
    ev |= 2;
  }
  if (S->k % P.interval == 0) outf = 1;
  if (S->x > S->tout) {
    outf = 1;
    S->tout = S->x + S->dtout;
  }
  S->outfield = outf;
  S->ev = ev;
  if (outf || ev) {
    S->snap = S->nsnap_used % P.nsnap;
    S->nsnap_used += 1;
  } else {
    S->snap = -1;
  }
  // stop controls (main_LH.f90:1425-1438), then the run's step limit
  int stop = 0;
  if (f.vmax > P.velmax) stop = HBI_STOP_VELMAX;
  else if (f.vmax < P.velmin) stop = HBI_STOP_VELMIN;
  else if (S->x > P.tmax) stop = HBI_STOP_TMAX;
  else if (S->k >= S->k_limit) stop = HBI_STOP_KLIMIT;
  if (stop && (!S->stop || S->stop == HBI_STOP_TLIMIT)) S->stop = stop;
  if (S->stop) {
    S->halted = 1;
    flags[0] = 1;
    flags[1] = 1;
  }
}

// fields of an output step into snapshot slot S->snap: vel, slip, sigma, tau
// and, at the end of an event, the event's slip |slip - islip|
__global__ void __launch_bounds__(256) cycle_snapshot_kernel(RkDev R, CycleConst P, const CycleState* S,
                                                             const double* __restrict__ vel,
                                                             const double* __restrict__ slip,
                                                             double* __restrict__ islip, double* __restrict__ snap) {
  if (!__ldcg(&S->accepted)) return;
  const int slot = __ldcg(&S->snap);
  if (slot < 0) return;
  const int ev = __ldcg(&S->ev);
  const int n = P.n;
  double* b = snap + (size_t)slot * 5 * n;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double s = slip[i];
    b[i] = vel[i];
    b[n + i] = s;
    b[2 * n + i] = R.y[3 * i + 2];
    b[3 * n + i] = R.y[3 * i + 1];
    if (ev & 2) b[4 * n + i] = fabs(s - islip[i]);
    if (ev & 1) islip[i] = s;
  }
}

// one record per attempt into the host-mapped ring
__global__ void cycle_record_kernel(CycleState* S, CycleState* ring, int nrec) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const long long j = S->launch;
  S->launch = j + 1;
  CycleState c = *S;
  c.launch = j;
  CycleState* d = ring + (j % nrec);
  const unsigned long long* src = (const unsigned long long*)&c;
  unsigned long long* dst = (unsigned long long*)d;
  for (size_t w = 0; w < sizeof(CycleState) / 8; w++) dst[w] = src[w];
  __threadfence_system();
  S->skipped = 0;
}

// start (or resume) a run: clear a resumable halt, set the run's limits, and
// shorten the pending step to the time limit
__global__ void cycle_resume_kernel(CycleState* S, int* flags, double* ctl, long long k_limit, double t_limit) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  if (S->stop == HBI_STOP_NONE || S->stop == HBI_STOP_KLIMIT || S->stop == HBI_STOP_TLIMIT) {
    S->stop = HBI_STOP_NONE;
    S->halted = 0;
    flags[0] = 0;
    flags[1] = flags[2];
  }
  S->k_limit = k_limit;
  S->t_limit = t_limit;
  if (t_limit <= S->x) {
    // already at (or past) the time limit: nothing to run
    S->stop = HBI_STOP_TLIMIT;
    S->halted = 1;
    flags[0] = 1;
    flags[1] = 1;
    return;
  }
  double h = S->h;
  if (S->clamped) {
    h = S->h_pending;
    S->clamped = 0;
  }
  if (S->x + h > t_limit) {
    S->h_pending = h;
    h = t_limit - S->x;
    S->clamped = 1;
  }
  S->h = h;
  ctl[0] = h;
}

static_assert(sizeof(CycleState) % 8 == 0, "record copy by 8-byte words");

// Fortran E editing (Ew.d, gfortran layout): [-]0.ddddE+xx right-justified
void fort_e(std::string& out, int w, int d, double v) {
  char buf[64], num[64];
  if (std::isnan(v)) {
    snprintf(buf, sizeof buf, "%*s", w, "NaN");
  } else if (std::isinf(v)) {
    snprintf(buf, sizeof buf, "%*s", w, v > 0 ? "Infinity" : "-Infinity");
  } else {
    int e10 = 0;
    std::string digits;
    const bool neg = std::signbit(v) && v != 0.0;
    if (v == 0.0) {
      digits.assign(d, '0');
    } else {
      snprintf(num, sizeof num, "%.*e", d - 1, std::fabs(v));  // d.ddd e+xx
      const char* p = num;
      digits.push_back(*p++);
      if (*p == '.') p++;
      while (*p && *p != 'e') digits.push_back(*p++);
      e10 = atoi(p + 1) + 1;
    }
    char ex[16];
    const int ae = e10 < 0 ? -e10 : e10;
    if (ae <= 99) snprintf(ex, sizeof ex, "E%c%02d", e10 < 0 ? '-' : '+', ae);
    else snprintf(ex, sizeof ex, "%c%03d", e10 < 0 ? '-' : '+', ae);
    std::string s = std::string(neg ? "-" : "") + "0." + digits + ex;
    snprintf(buf, sizeof buf, "%*s", w, s.c_str());
  }
  out += buf;
}

void fort_f(std::string& out, int w, int d, double v) {
  char buf[64];
  snprintf(buf, sizeof buf, "%*.*f", w, d, v);
  out += buf;
}

void fort_i(std::string& out, int w, long long v) {
  char buf[32];
  if (w > 0) snprintf(buf, sizeof buf, "%*lld", w, v);
  else snprintf(buf, sizeof buf, "%lld", v);
  out += buf;
}

}  // namespace
}  // namespace hbi

using namespace hbi;

static constexpr int kPropFloats =
    proposer_weights(HBI_PROPOSER_NIN, HBI_PROPOSER_HID) + 2 * HBI_PROPOSER_NIN + 2;

struct hbi_cycle_s {
  hbi_rk* rk = nullptr;
  RkView V{};
  RkDev R{};
  MatDev m_first[2]{}, m_rest[2]{};
  CycleConst P{};
  hbi_cycle_params prm{};
  ProposerDev M{};
  cudaStream_t st = nullptr;
  CycleState* dS = nullptr;
  int* dflags = nullptr;
  MonPart* dpart = nullptr;
  double *dvel = nullptr, *dslip = nullptr, *dds = nullptr, *dislip = nullptr, *dsnap = nullptr;
  float* dprop = nullptr;
  CycleState* hring = nullptr;  // host-mapped
  CycleState* dring = nullptr;
  double* hsnap = nullptr;      // pinned staging, one per snapshot slot
  int G = 1;
  cudaGraphExec_t gexec = nullptr;
  static constexpr int kMaxInflight = 16;
  cudaEvent_t ev[kMaxInflight] = {};
  cudaEvent_t snap_ev[kMaxInflight + 2] = {};
  struct Pending {
    CycleState rec;
    int slot;
  };
  std::deque<Pending> pending;
  std::vector<hbi_event> events;
  std::vector<double> trace;
  long long nlaunch = 0;
  long long attempts = 0;
  long long kend = -1;  // a restart does not rewrite monitor lines up to this step
  CycleState last{};
  std::FILE *fmon = nullptr, *ftime = nullptr, *fevent = nullptr;
  std::FILE* ffield[5] = {};
  std::chrono::steady_clock::time_point t1;
};

namespace {

void close_files(hbi_cycle* c) {
  for (std::FILE** f : {&c->fmon, &c->ftime, &c->fevent})
    if (*f) {
      std::fclose(*f);
      *f = nullptr;
    }
  for (auto& f : c->ffield)
    if (f) {
      std::fclose(f);
      f = nullptr;
    }
}

int cfail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  return set_error(code, buf);
}

#define CCK(x)                                                                                       \
  do {                                                                                               \
    cudaError_t e_ = (x);                                                                            \
    if (e_ != cudaSuccess) return cfail(HBI_ERR_CUDA, "%s: %s (%s:%d)", #x, cudaGetErrorString(e_), __FILE__, __LINE__); \
  } while (0)

double wall_since(const std::chrono::steady_clock::time_point& t) {
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t).count();
}

// monitor line (main_LH.f90:1489-1493): '(i7,f19.4,7e16.5,i4,f16.4)'
void write_monitor(hbi_cycle* c, const CycleState& s, double errmax, double dtdid, int nrjct) {
  if (!c->fmon || s.k <= c->kend) return;
  std::string l;
  fort_i(l, 7, s.k);
  fort_f(l, 19, 4, s.x);
  fort_e(l, 16, 5, std::log10(s.mvel));
  fort_e(l, 16, 5, s.meanslip);
  fort_e(l, 16, 5, s.meanmu);
  fort_e(l, 16, 5, s.maxnorm);
  fort_e(l, 16, 5, s.minnorm);
  fort_e(l, 16, 5, errmax);
  fort_e(l, 16, 5, dtdid);
  fort_i(l, 4, nrjct);
  fort_f(l, 16, 4, wall_since(c->t1));
  l += "\n";
  std::fputs(l.c_str(), c->fmon);
}

void write_time(hbi_cycle* c, long long k, double x) {
  if (!c->ftime) return;
  std::string l;
  fort_i(l, 7, k);
  fort_f(l, 19, 4, x);
  l += "\n";
  std::fputs(l.c_str(), c->ftime);
}

// fields of one snapshot (output_field, main_LH.f90:1518-1559; EQslip :1613-1630)
void write_snapshot(hbi_cycle* c, const CycleState& rec, const double* b) {
  const int n = c->P.n;
  if (rec.outfield) {
    write_time(c, rec.k, rec.x);
    for (int f = 0; f < 4; f++)
      if (c->ffield[f]) std::fwrite(b + (size_t)f * n, sizeof(double), n, c->ffield[f]);
    if (c->fmon) std::fflush(c->fmon);
  }
  if ((rec.ev & 2) && c->ffield[4]) std::fwrite(b + 4 * (size_t)n, sizeof(double), n, c->ffield[4]);
}

int flush_pending(hbi_cycle* c, bool wait_all) {
  while (!c->pending.empty()) {
    auto& p = c->pending.front();
    if (wait_all) {
      CCK(cudaEventSynchronize(c->snap_ev[p.slot]));
    } else {
      const cudaError_t q = cudaEventQuery(c->snap_ev[p.slot]);
      if (q == cudaErrorNotReady) break;
      CCK(q);
    }
    write_snapshot(c, p.rec, c->hsnap + (size_t)p.slot * 5 * c->P.n);
    c->pending.pop_front();
  }
  return HBI_OK;
}

void enqueue_attempt(hbi_cycle* c) {
  const RkDev& R = c->R;
  const int nmat = c->V.nmat, sm = c->V.sm;
  cudaStream_t st = c->st;
  launch_rk_prepare(R, st);
  for (int s = 0; s < 6; s++) {
    const double* xin = s == 0 ? R.x0 : R.xb[s & 1];
    double* xout = R.xb[(s + 1) & 1];
    const MatDev* m = s == 0 ? c->m_first : c->m_rest;
    launch_phase1(m, nmat, xin, sm, st);
    launch_phase2(m, nmat, xin, sm, st);
    launch_phase3_rk(c->m_rest, nmat, R, s, xout, st);
  }
  cycle_control_kernel<<<1, 256, 0, st>>>(R, c->P, c->dS, c->dflags, c->M, c->V.mats[0].err,
                                          nmat == 2 ? c->V.mats[1].err : nullptr);
  cycle_update_kernel<<<c->G, 256, 0, st>>>(R, c->P, c->dS, c->dflags, c->dvel, c->dslip, c->dds, c->dpart, 0);
  cycle_snapshot_kernel<<<c->G, 256, 0, st>>>(R, c->P, c->dS, c->dvel, c->dslip, c->dislip, c->dsnap);
  cycle_record_kernel<<<1, 32, 0, st>>>(c->dS, c->dring, c->P.nrec);
}

int launch_one(hbi_cycle* c) {
  const int w = (int)(c->nlaunch % c->prm.inflight);
  CCK(cudaGraphLaunch(c->gexec, c->st));
  CCK(cudaEventRecord(c->ev[w], c->st));
  c->nlaunch++;
  return HBI_OK;
}

// host side of one record: monitor line, snapshot copy, event line, trace
int process_record(hbi_cycle* c, const CycleState& r) {
  if (r.skipped) return HBI_OK;
  c->attempts++;
  c->trace.insert(c->trace.end(), {(double)r.k, r.x, r.h_try, r.errmax, (double)r.accepted, r.mvel, r.hnext,
                                   (double)r.nrjct});
  if (!r.accepted) return HBI_OK;
  write_monitor(c, r, r.errmax, r.hdid, r.nrjct);
  if (r.ev & 2) {
    hbi_event e{};
    e.id = r.eventcount;
    e.hypoloc = r.hypoloc;
    e.k = r.k;
    e.onset = r.onset;
    e.end = r.x;
    e.moment = r.moment;
    e.mw = (std::log10(r.moment * c->prm.rigid * c->P.sg) + 5.9) / 1.5;
    c->events.push_back(e);
    if (c->fevent) {
      // '(i0,i8,f17.2,f14.4,i8)' (main_LH.f90:1375)
      std::string l;
      fort_i(l, 0, e.id);
      fort_i(l, 8, e.k);
      fort_f(l, 17, 2, e.onset);
      fort_f(l, 14, 4, e.mw);
      fort_i(l, 8, e.hypoloc);
      l += "\n";
      std::fputs(l.c_str(), c->fevent);
      std::fflush(c->fevent);
    }
  }
  if (r.snap >= 0 && c->prm.outdir) {
    // the slot is not rewritten before `inflight` + 2 more snapshots, and the
    // attempts already enqueued make at most `inflight` - 1 of them
    for (const auto& p : c->pending)
      if (p.slot == r.snap) {
        int rc = flush_pending(c, true);
        if (rc) return rc;
        break;
      }
    const size_t bytes = sizeof(double) * 5 * (size_t)c->P.n;
    CCK(cudaMemcpyAsync(c->hsnap + (size_t)r.snap * 5 * c->P.n, c->dsnap + (size_t)r.snap * 5 * c->P.n, bytes,
                        cudaMemcpyDeviceToHost, c->st));
    CCK(cudaEventRecord(c->snap_ev[r.snap], c->st));
    c->pending.push_back({r, r.snap});
  }
  return HBI_OK;
}

}  // namespace

extern "C" int hbi_cycle_free(hbi_cycle* c) {
  if (!c) return HBI_OK;
  if (c->st) cudaStreamSynchronize(c->st);
  flush_pending(c, true);
  close_files(c);
  if (c->gexec) cudaGraphExecDestroy(c->gexec);
  for (auto& e : c->ev)
    if (e) cudaEventDestroy(e);
  for (auto& e : c->snap_ev)
    if (e) cudaEventDestroy(e);
  cudaFree(c->dS);
  cudaFree(c->dflags);
  cudaFree(c->dpart);
  cudaFree(c->dvel);
  cudaFree(c->dslip);
  cudaFree(c->dds);
  cudaFree(c->dislip);
  cudaFree(c->dsnap);
  cudaFree(c->dprop);
  if (c->hring) cudaFreeHost(c->hring);
  if (c->hsnap) cudaFreeHost(c->hsnap);
  if (c->st) cudaStreamDestroy(c->st);
  delete c;
  return HBI_OK;
}

namespace {
// where a restarted loop resumes (main_LH.f90:836-957)
struct RestartPoint {
  long long k, kend;   // steps done; last step already in the monitor file
  double x, h;
  std::vector<double> slip;
};

int cycle_create_impl(hbi_cycle** out, hbi_rk* rk, const double* vel, const double* ds, const hbi_cycle_params* p,
                      const RestartPoint* rs);
}  // namespace

extern "C" int hbi_cycle_create(hbi_cycle** out, hbi_rk* rk, const double* vel, const double* ds,
                                const hbi_cycle_params* p) {
  return cycle_create_impl(out, rk, vel, ds, p, nullptr);
}

namespace {
int cycle_create_impl(hbi_cycle** out, hbi_rk* rk, const double* vel, const double* ds, const hbi_cycle_params* p,
                      const RestartPoint* rs) {
  if (!out || !rk || !vel || !ds || !p) return cfail(HBI_ERR_ARG, "hbi_cycle_create: null argument");
  if (p->inflight < 1 || p->inflight > hbi_cycle_s::kMaxInflight)
    return cfail(HBI_ERR_ARG, "inflight must be in 1..%d", hbi_cycle_s::kMaxInflight);
  if (!(p->eps_r > 0) || !(p->dtinit > 0)) return cfail(HBI_ERR_ARG, "eps_r and dtinit must be positive");
  hbi_cycle* c = new hbi_cycle_s();
  c->rk = rk;
  c->prm = *p;
  int rc = rk_view(rk, &c->V);
  if (rc) {
    delete c;
    return rc;
  }
  // the loop works on a stream of its own, after whatever the RK handle has
  // enqueued: freeing the loop then never touches the RK handle's stream
  if (cudaStreamSynchronize((cudaStream_t)hbi_rk_stream(rk)) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking) != cudaSuccess) {
    c->st = nullptr;
    delete c;
    return cfail(HBI_ERR_CUDA, "hbi_cycle_create: stream");
  }
  const int n = c->V.n;
  CycleConst& P = c->P;
  P.n = n;
  P.nsnap = p->outdir ? p->inflight + 2 : 1;
  P.nrec = 64;
  P.eps = p->eps_r;
  P.dtmax = p->dtmax;
  P.tmax = p->tmax;
  P.velth = p->velth;
  P.velmax = p->velmax;
  P.velmin = p->velmin;
  P.dtout_inter = p->dtout_inter;
  P.dtout_co = p->dtout_co;
  P.interval = p->interval > 0 ? p->interval : (p->nstep > 0 ? p->nstep : 1LL << 62);
  // sg: total area, summed in cluster order as the reference does
  double sg = 0.0;
  for (int i = 0; i < n; i++) sg += ds[i];
  P.sg = sg;
  int dev = 0, sm = 152;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sm, cudaDevAttrMultiProcessorCount, dev);
  c->G = std::max(1, std::min((n + 255) / 256, 2 * sm));
  auto fail_free = [&](int code, const char* what) {
    hbi_cycle_free(c);
    return cfail(code, "hbi_cycle_create: %s", what);
  };
  if (cudaMalloc(&c->dS, sizeof(CycleState)) != cudaSuccess || cudaMalloc(&c->dflags, 4 * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&c->dpart, sizeof(MonPart) * c->G) != cudaSuccess ||
      cudaMalloc(&c->dvel, sizeof(double) * n) != cudaSuccess || cudaMalloc(&c->dslip, sizeof(double) * n) != cudaSuccess ||
      cudaMalloc(&c->dds, sizeof(double) * n) != cudaSuccess || cudaMalloc(&c->dislip, sizeof(double) * n) != cudaSuccess ||
      cudaMalloc(&c->dsnap, sizeof(double) * 5 * (size_t)n * P.nsnap) != cudaSuccess ||
      cudaMalloc(&c->dprop, sizeof(float) * kPropFloats) != cudaSuccess ||
      cudaHostAlloc(&c->hring, sizeof(CycleState) * P.nrec, cudaHostAllocMapped) != cudaSuccess ||
      (p->outdir && cudaMallocHost(&c->hsnap, sizeof(double) * 5 * (size_t)n * P.nsnap) != cudaSuccess))
    return fail_free(HBI_ERR_NOMEM, "allocation");
  if (cudaHostGetDevicePointer((void**)&c->dring, c->hring, 0) != cudaSuccess)
    return fail_free(HBI_ERR_CUDA, "mapped record ring");
  memset(c->hring, 0, sizeof(CycleState) * P.nrec);
  for (auto& e : c->ev)
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return fail_free(HBI_ERR_CUDA, "events");
  for (auto& e : c->snap_ev)
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return fail_free(HBI_ERR_CUDA, "events");
  c->M.w = c->dprop;
  c->M.nin = HBI_PROPOSER_NIN;
  c->M.hid = HBI_PROPOSER_HID;
  // the RK handle's device state, with the loop's flags: [0] halted,
  // [1] halted or retrying, [2] retrying
  c->R = c->V.R;
  c->R.flags = c->dflags;
  for (int i = 0; i < 2; i++) {
    c->m_first[i] = c->V.mats[i];
    c->m_first[i].skip = c->dflags + 1;
    c->m_rest[i] = c->V.mats[i];
    c->m_rest[i].skip = c->dflags;
  }
  CycleState s0{};
  s0.x = rs ? rs->x : 0.0;
  s0.k = rs ? rs->k : 0;
  s0.h = rs ? rs->h : p->dtinit;
  c->kend = rs ? rs->kend : -1;
  s0.dtout = p->dtout_inter;
  s0.tout = s0.dtout;
  s0.t_limit = INFINITY;
  s0.k_limit = p->nstep > 0 ? p->nstep : (1LL << 62);
  s0.snap = -1;
  s0.hist_e1 = 0.5;
  s0.hist_h1 = s0.h;
  s0.learned = 0;
  const int zf[4] = {0, 0, 0, 0};
  const double ctl2[2] = {s0.h, p->eps_r};
  cudaStream_t st = c->st;
  if (cudaMemcpyAsync(c->dS, &s0, sizeof s0, cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(c->dflags, zf, sizeof zf, cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(c->R.ctl, ctl2, sizeof ctl2, cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(c->dvel, vel, sizeof(double) * n, cudaMemcpyHostToDevice, st) != cudaSuccess ||
      (rs ? cudaMemcpyAsync(c->dslip, rs->slip.data(), sizeof(double) * n, cudaMemcpyHostToDevice, st)
          : cudaMemsetAsync(c->dslip, 0, sizeof(double) * n, st)) != cudaSuccess ||
      cudaMemsetAsync(c->dislip, 0, sizeof(double) * n, st) != cudaSuccess ||
      cudaMemcpyAsync(c->dds, ds, sizeof(double) * n, cudaMemcpyHostToDevice, st) != cudaSuccess)
    return fail_free(HBI_ERR_CUDA, "upload");
  // k = 0: monitors of the initial state (main_LH.f90:1144-1183)
  cycle_update_kernel<<<c->G, 256, 0, st>>>(c->R, P, c->dS, c->dflags, c->dvel, c->dslip, c->dds, c->dpart, 1);
  CycleState s{};
  if (cudaMemcpyAsync(&s, c->dS, sizeof s, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return fail_free(HBI_ERR_CUDA, "initial monitors");
  // the proposer's slip-rate history starts from the initial state
  s.hist_v1 = s.hist_v2 = s.mvel;
  if (cudaMemcpyAsync(c->dS, &s, sizeof s, cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return fail_free(HBI_ERR_CUDA, "initial monitors");
  c->last = s;
  if (p->outdir) {
    auto open = [&](const char* stem, const char* mode) {
      char fn[1024];
      snprintf(fn, sizeof fn, "%s/%s%d.dat", p->outdir, stem, p->number);
      return std::fopen(fn, mode);
    };
    // a restart appends to the files of the run it continues (EQslip restarts)
    c->fmon = open("monitor", rs ? "a" : "w");
    c->ftime = open("time", rs ? "a" : "w");
    c->fevent = open("event", rs ? "a" : "w");
    const char* stems[5] = {"vel", "slip", "sigma", "tau", "EQslip"};
    for (int f = 0; f < 5; f++) c->ffield[f] = open(stems[f], (rs && f < 4) ? "ab" : "wb");
    if (!c->fmon || !c->ftime || !c->fevent || !c->ffield[0] || !c->ffield[4])
      return fail_free(HBI_ERR_ARG, "cannot open output files");
  }
  c->t1 = std::chrono::steady_clock::now();
  if (p->outdir && !rs) {
    // k = 0 outputs: time line, monitor line, fields (vel, slip=0, sigma, tau)
    write_time(c, 0, 0.0);
    write_monitor(c, s, 0.0, 0.0, 0);
    std::vector<double> y(3 * (size_t)n), b(4 * (size_t)n);
    if (cudaMemcpy(y.data(), c->R.y, sizeof(double) * y.size(), cudaMemcpyDeviceToHost) != cudaSuccess)
      return fail_free(HBI_ERR_CUDA, "initial state");
    for (int i = 0; i < n; i++) {
      b[i] = vel[i];
      b[n + i] = 0.0;
      b[2 * (size_t)n + i] = y[3 * (size_t)i + 2];
      b[3 * (size_t)n + i] = y[3 * (size_t)i + 1];
    }
    for (int f = 0; f < 4; f++)
      if (c->ffield[f]) std::fwrite(b.data() + (size_t)f * n, sizeof(double), n, c->ffield[f]);
  }
  // the attempt graph
  cudaGraph_t g;
  if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
    return fail_free(HBI_ERR_CUDA, "capture");
  enqueue_attempt(c);
  if (cudaStreamEndCapture(st, &g) != cudaSuccess) return fail_free(HBI_ERR_CUDA, "capture");
  const cudaError_t ie = cudaGraphInstantiate(&c->gexec, g, 0);
  cudaGraphDestroy(g);
  if (ie != cudaSuccess) return fail_free(HBI_ERR_CUDA, "graph instantiate");
  *out = c;
  return HBI_OK;
}

// one Fortran E/F field: also accepts the exponent without its letter
// ("0.12345-100") that Ew.d writes for three-digit exponents
bool fort_read(const char*& p, double* v) {
  while (*p == ' ' || *p == '\t') p++;
  if (!*p || *p == '\n') return false;
  char* end = nullptr;
  double d = strtod(p, &end);
  if (end == p) return false;
  if ((*end == '+' || *end == '-') && end[1] >= '0' && end[1] <= '9') {
    char* e2 = nullptr;
    const long ex = strtol(end, &e2, 10);
    d *= pow(10.0, (double)ex);
    end = e2;
  }
  p = end;
  *v = d;
  return true;
}
}  // namespace

extern "C" int hbi_restart_point(const char* monitor_path, long long interval, long long* k, double* x,
                                 double* dtnxt, long long* kend) {
  if (!monitor_path || !k || !x || !dtnxt || interval < 1) return cfail(HBI_ERR_ARG, "hbi_restart_point: arguments");
  std::FILE* f = std::fopen(monitor_path, "r");
  if (!f) return cfail(HBI_ERR_ARG, "hbi_restart_point: cannot open %s", monitor_path);
  char line[1024];
  long long kk = -1, klast = -1;
  double xx = 0, dn = 0;
  while (std::fgets(line, sizeof line, f)) {
    const char* q = line;
    double v[11];
    int nv = 0;
    while (nv < 11 && fort_read(q, &v[nv])) nv++;
    if (nv < 10) continue;
    const long long kl = (long long)v[0];
    klast = kl;
    if (kl % interval == 0) {
      // main_LH.f90:841-845: x and the next trial step of the last line
      // whose step is a multiple of the output interval
      kk = kl;
      xx = v[1];
      const double errmax = v[7], dtdid = v[8];
      dn = std::min(2 * dtdid, (double)0.9f * dtdid * pow(errmax, (double)-0.2f));
    }
  }
  std::fclose(f);
  if (kk < 0) return cfail(HBI_ERR_STATE, "hbi_restart_point: no step at a multiple of the interval in %s", monitor_path);
  *k = kk;
  *x = xx;
  *dtnxt = dn;
  if (kend) *kend = klast;
  return HBI_OK;
}

extern "C" int hbi_cycle_restart(hbi_cycle** out, hbi_rk* rk, const double* ds, const hbi_cycle_params* p) {
  if (!out || !rk || !ds || !p || !p->outdir) return cfail(HBI_ERR_ARG, "hbi_cycle_restart: arguments");
  RkView V{};
  int rc = rk_view(rk, &V);
  if (rc) return rc;
  const int n = V.n;
  char fn[1024];
  snprintf(fn, sizeof fn, "%s/monitor%d.dat", p->outdir, p->number);
  const long long interval = p->interval > 0 ? p->interval : (p->nstep > 0 ? p->nstep : 1LL << 62);
  RestartPoint rs;
  long long k0;
  rc = hbi_restart_point(fn, interval, &k0, &rs.x, &rs.h, &rs.kend);
  if (rc) return rc;
  rs.k = k0;
  // the last snapshot of each field file (main_LH.f90:867-897)
  std::vector<double> fld[4];
  const char* stems[4] = {"vel", "slip", "sigma", "tau"};
  for (int f = 0; f < 4; f++) {
    snprintf(fn, sizeof fn, "%s/%s%d.dat", p->outdir, stems[f], p->number);
    std::FILE* fp = std::fopen(fn, "rb");
    if (!fp) return cfail(HBI_ERR_ARG, "hbi_cycle_restart: cannot open %s", fn);
    std::fseek(fp, 0, SEEK_END);
    const long sz = std::ftell(fp);
    if (sz < (long)sizeof(double) * n) {
      std::fclose(fp);
      return cfail(HBI_ERR_STATE, "hbi_cycle_restart: %s holds no snapshot", fn);
    }
    fld[f].resize(n);
    std::fseek(fp, sz - (long)sizeof(double) * n, SEEK_SET);
    const size_t got = std::fread(fld[f].data(), sizeof(double), n, fp);
    std::fclose(fp);
    if (got != (size_t)n) return cfail(HBI_ERR_STATE, "hbi_cycle_restart: short read of %s", fn);
  }
  rs.slip = fld[1];
  // psi from the slip rate and stresses (main_LH.f90:899)
  std::vector<double> a(n), y(3 * (size_t)n);
  if (cudaMemcpy(a.data(), V.R.a, sizeof(double) * n, cudaMemcpyDeviceToHost) != cudaSuccess)
    return cfail(HBI_ERR_CUDA, "hbi_cycle_restart: a");
  const double vref = V.R.vref;
  for (int i = 0; i < n; i++) {
    const double vel = fld[0][i], sig = fld[2][i], tau = fld[3][i];
    y[3 * (size_t)i] = a[i] * log(2 * vref / vel * sinh(tau / sig / a[i]));
    y[3 * (size_t)i + 1] = tau;
    y[3 * (size_t)i + 2] = sig;
  }
  rc = hbi_rk_set_state(rk, y.data());
  if (rc) return rc;
  return cycle_create_impl(out, rk, fld[0].data(), ds, p, &rs);
}

extern "C" int hbi_cycle_run(hbi_cycle* c, long long k_limit, double t_limit, hbi_cycle_status* out) {
  if (!c) return cfail(HBI_ERR_ARG, "null");
  const auto t0 = std::chrono::steady_clock::now();
  const long long kl = k_limit > 0 ? k_limit : (c->prm.nstep > 0 ? c->prm.nstep : (1LL << 62));
  const double tl = t_limit > 0 ? t_limit : INFINITY;
  if (c->last.stop == HBI_STOP_DEVICE)
    return cfail(HBI_ERR_DEVICE, "hbi_cycle_run: the loop stopped on a device error and cannot continue");
  if (c->last.stop && c->last.stop != HBI_STOP_KLIMIT && c->last.stop != HBI_STOP_TLIMIT) {
    // a stop control already ended the loop
    if (out) {
      memset(out, 0, sizeof *out);
      out->stop = c->last.stop;
      out->k = c->last.k;
      out->x = c->last.x;
    }
    return HBI_OK;
  }
  cycle_resume_kernel<<<1, 1, 0, c->st>>>(c->dS, c->dflags, c->R.ctl, kl, tl);
  CCK(cudaGetLastError());
  const int W = c->prm.inflight;
  const long long first = c->nlaunch;
  for (int i = 0; i < W; i++) {
    int rc = launch_one(c);
    if (rc) return rc;
  }
  long long j = first;
  bool halted = false;
  long long rej0 = 0;
  for (;;) {
    CCK(cudaEventSynchronize(c->ev[j % W]));
    const CycleState r = c->hring[j % c->P.nrec];
    if (r.launch != j) return cfail(HBI_ERR_STATE, "record ring out of step (%lld != %lld)", r.launch, j);
    int rc = process_record(c, r);
    if (rc) return rc;
    if (!r.skipped) c->last = r;
    rej0 += (!r.skipped && !r.accepted) ? 1 : 0;
    if (r.halted) halted = true;
    j++;
    if (!halted) {
      rc = launch_one(c);
      if (rc) return rc;
    }
    if (j == c->nlaunch) break;
    rc = flush_pending(c, false);
    if (rc) return rc;
  }
  CCK(cudaStreamSynchronize(c->st));
  int rc = flush_pending(c, true);
  if (rc) return rc;
  for (std::FILE* f : {c->fmon, c->ftime, c->fevent})
    if (f) std::fflush(f);
  if (out) {
    const CycleState& s = c->last;
    out->k = s.k;
    out->attempts = c->attempts;
    out->rejected = s.rejected;
    out->x = s.x;
    out->hnext = s.h;
    out->errmax = s.errmax;
    out->dtdid = s.hdid;
    out->mvel = s.mvel;
    out->meanslip = s.meanslip;
    out->meanmu = s.meanmu;
    out->maxnorm = s.maxnorm;
    out->minnorm = s.minnorm;
    out->nrjct = s.nrjct;
    out->events = (int)c->events.size();
    out->slipping = s.slipping;
    out->stop = s.stop;
    out->wall_s = wall_since(t0);
  }
  if (c->last.stop == HBI_STOP_UNDERFLOW) return cfail(HBI_ERR_CONVERGE, "Runge-Kutta step size underflow at x=%.17g", c->last.x);
  if (c->last.stop == HBI_STOP_DEVICE) {
    // clear the operators' error words and arrival counters for their next use
    for (int k = 0; k < c->V.nmat; k++)
      if (take_device_error(c->V.mats[k]) < 0) return cfail(HBI_ERR_CUDA, "hbi_cycle_run: device error reset");
    return cfail(HBI_ERR_DEVICE, "hbi_cycle_run: a product kernel gave up waiting for a bulk copy at step %lld; "
                 "the loop stopped (the operators' device state has been reset)", c->last.k + 1);
  }
  return HBI_OK;
}

extern "C" int hbi_cycle_fields(hbi_cycle* c, double* vel, double* slip) {
  if (!c) return cfail(HBI_ERR_ARG, "null");
  CCK(cudaStreamSynchronize(c->st));
  if (vel) CCK(cudaMemcpy(vel, c->dvel, sizeof(double) * c->P.n, cudaMemcpyDeviceToHost));
  if (slip) CCK(cudaMemcpy(slip, c->dslip, sizeof(double) * c->P.n, cudaMemcpyDeviceToHost));
  return HBI_OK;
}

extern "C" int hbi_cycle_events(hbi_cycle* c, hbi_event* ev, int max, int* count) {
  if (!c || !count) return cfail(HBI_ERR_ARG, "null");
  *count = (int)c->events.size();
  if (ev)
    for (int i = 0; i < std::min(max, *count); i++) ev[i] = c->events[i];
  return HBI_OK;
}

extern "C" int hbi_cycle_trace(hbi_cycle* c, double* rec, long long max, long long* count) {
  if (!c || !count) return cfail(HBI_ERR_ARG, "null");
  const long long nr = (long long)(c->trace.size() / 8);
  *count = nr;
  if (rec) memcpy(rec, c->trace.data(), sizeof(double) * 8 * (size_t)std::min(max, nr));
  return HBI_OK;
}

extern "C" int hbi_cycle_set_proposer(hbi_cycle* c, const float* w) {
  if (!c) return cfail(HBI_ERR_ARG, "null");
  CCK(cudaStreamSynchronize(c->st));
  if (w) CCK(cudaMemcpy(c->dprop, w, sizeof(float) * kPropFloats, cudaMemcpyHostToDevice));
  const int on = w ? 1 : 0;
  CCK(cudaMemcpy((char*)c->dS + offsetof(CycleState, learned), &on, sizeof on, cudaMemcpyHostToDevice));
  return HBI_OK;
}

extern "C" int hbi_cycle_proposer_size(int* nin, int* hid, int* nfloats) {
  if (nin) *nin = HBI_PROPOSER_NIN;
  if (hid) *hid = HBI_PROPOSER_HID;
  if (nfloats) *nfloats = kPropFloats;
  return HBI_OK;
}
