/*
 * hbi_gpu.h -- C ABI of the GB300 implementation of HBI's per-step hot path.
 *
 * Each entry point replaces one HACApK / HBI routine that the Fortran driver
 * (main_LH.f90) calls; the comment on each names the reference routine by
 * file:line.  All functions return 0 (HBI_OK) or a negative HBI_ERR_* code and
 * never abort; hbi_last_error() returns a message for the calling thread.
 * Arrays are plain C arrays; "cluster order" means the lattice-vector order of
 * HACApK (element lodc(i) of the global numbering sits at position i), which
 * is the order every state array of the reference driver lives in.
 * Integer element ids that the reference keeps 1-based (lod, lodc, leaf starts)
 * stay 1-based.
 *
 * Threading: a handle is used by one host thread at a time.  Every handle
 * owns its device memory and issues work on its own CUDA stream; the *_dev
 * variants take device pointers and a stream and do not synchronise.
 */
#ifndef HBI_GPU_H
#define HBI_GPU_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

#define HBI_OK 0
#define HBI_ERR_ARG (-1)      /* invalid argument */
#define HBI_ERR_CUDA (-2)     /* CUDA runtime error (see hbi_last_error) */
#define HBI_ERR_NOMEM (-3)    /* device or host allocation failed */
#define HBI_ERR_STATE (-4)    /* call out of order (e.g. construct before generate) */
#define HBI_ERR_CONVERGE (-5) /* Runge-Kutta step size underflow (reference: stop) */
#define HBI_ERR_LIMIT (-6)    /* a size limit of this entry point was exceeded */
#define HBI_ERR_DEVICE (-7)   /* a product kernel gave up a bounded wait for one of its bulk
                                 copies: the results of the calls since the last check are
                                 invalid; the operator's device state has been reset */

/* problem kinds: st_bemv%problem of m_HACApK_calc_entry_ij.f90:24-90 */
#define HBI_2DVS 1 /* 2D antiplane, half space (matels2dpa_ij :685-695)   */
#define HBI_3DPH 2 /* 3D rectangles, Okada half space (okada_ij :1065-1145) */
#define HBI_3DNR 3 /* 3D rectangles, Okada full space                    */
#define HBI_3DNT 4 /* 3D triangles, TDstressFS full space (matel3dn_ij :802-851) */
#define HBI_2DPH 5 /* 2D plane strain, half space; also '2dnh' (matel2dph2_ij :92-166) */
#define HBI_2DN 6  /* 2D plane strain, full space (tensor2d_ij :300-339) */
#define HBI_3DHT 7 /* 3D triangles, TDstressHS half space (matel3dh_ij :852-898) */

/* factor storage of the matvec operator */
#define HBI_STORE_F64 0
#define HBI_STORE_F32 1
#define HBI_STORE_BF16 2

/* st_HACApK_calc_entry (m_HACApK_calc_entry_ij.f90:7-19): geometry in the
 * global (input) numbering, all arrays of length nd; unused ones may be NULL. */
typedef struct {
  int problem;  /* HBI_2DVS .. HBI_3DHT */
  int nd;
  char v;       /* 's' shear or 'n' normal traction (st_bemv%v) */
  char md;      /* 's' slip along rake (st_bemv%md); only 's' is supported */
  const double *xcol, *ycol, *zcol;
  const double *xel, *xer;                      /* 2dvs, 2dph, 2dn element ends */
  const double *ang, *angd, *dsl, *dsd, *rake;  /* okada; ang also 2D; rake also triangles (radians) */
  double w;                                     /* okada length scale (ds0) */
  const double *xs1, *xs2, *xs3, *ys1, *ys2, *ys3, *zs1, *zs2, *zs3; /* triangles */
  const double *ev11, *ev12, *ev13, *ev21, *ev22, *ev23, *ev31, *ev32, *ev33;
  const double *yel, *yer;                      /* 2dph / 2dn element ends (with xel, xer) */
} hbi_bemv;

typedef struct hbi_ctl_s hbi_ctl;           /* st_HACApK_lcontrol */
typedef struct hbi_leafmtxp_s hbi_leafmtxp; /* st_HACApK_leafmtxp (filled leaves) */
typedef struct hbi_lhp_s hbi_lhp;           /* st_HACApK_LHp (lattice matvec operator) */
typedef struct hbi_rk_s hbi_rk;             /* RK45 state of the derivs/rkck/rkqs loop */

const char* hbi_last_error(void);
int hbi_version(void);
/* select the CUDA device that subsequent hbi_init calls on this thread bind */
int hbi_set_device(int device);

/* HACApK_init (m_HACApK_base.f90:246-345): control block with the default
 * param(1:100) of a one-rank run (param(43)=1).  Binds the current device. */
int hbi_init(int nd, hbi_ctl** ctl);
/* HACApK_param_set (m_HACApK_base.f90:348-382): copies param(1:100) */
int hbi_param_set(hbi_ctl* ctl, const double* param100);
int hbi_param_get(const hbi_ctl* ctl, double* param100);
/* HACApK_finalize (m_HACApK_base.f90:385-393) */
int hbi_finalize(hbi_ctl* ctl);

/* HACApK_generate (m_HACApK_use.f90:133-260): cluster tree, admissibility and
 * leaf list (bit-exact with HACApK), then ACA+ for admissible leaves and the
 * dense near field on the GPU in FP64.  coord is coord(nd,3) column-major;
 * ztol is eps_h.  The tree is stored in ctl (st_ctl%lod). */
int hbi_generate(hbi_leafmtxp** st_leafmtxp, const hbi_bemv* st_bemv, hbi_ctl* st_ctl,
                 const double* coord, double ztol);
/* The structure half of HACApK_generate, host only (no GPU needed): cluster
 * tree, admissibility and sorted leaf list of generate_frame_blrleaf
 * (m_HACApK_base.f90:649-951) for one rank.  param100 may be NULL (defaults).
 * lod receives lod(1:nd); call with leaves6 == NULL to get *nleaf, then again
 * with room for 6 * *nleaf ints (ltmtx, kt=0, nstrtl, ndl, nstrtt, ndt). */
int hbi_cluster_structure(int nd, const double* coord, const double* param100, int* lod, int* nleaf,
                          int* leaves6);
/* HACApK_free_leafmtxp (m_HACApK_base.f90:3084) */
int hbi_free_leafmtxp(hbi_leafmtxp* lf);

/* HACApK_construct_LH (m_HACApK_use.f90:263-366) with HACApK_contiguous
 * (m_HACApK_base.f90:3652-3740): packs the filled leaves into the matvec
 * operator with the given factor storage (HBI_STORE_*).  The operator keeps
 * no reference to lf, which may be freed afterwards. */
int hbi_construct_lh(hbi_lhp** st_LHp, const hbi_leafmtxp* lf, hbi_ctl* st_ctl, int storage);
int hbi_free_lh(hbi_lhp* lh);

/* Sharding of the product over ranks.  The reference distributes lattice
 * blocks over a 2-D MPI process grid and combines each rank's partial row
 * sums by a row reduce and a column broadcast (m_HACApK_solve.f90:278-314).
 * Here the leaves are dealt to nranks ranks by factor elements, largest
 * first to the least-loaded rank (host only, no GPU): owner[leaf] receives
 * the rank, elems_per_rank[nranks] the load of each (may be NULL).  A rank's
 * operator (hbi_construct_lh_part) holds only its leaves, so its product is
 * a partial au; the sum of the ranks' partials -- one all-reduce of ndc
 * doubles per product -- is au. */
int hbi_partition_leaves(int nleaf, const int* leaves6, int nranks, int32_t* owner, int64_t* elems_per_rank);
/* hbi_construct_lh over the leaves with owner[leaf] == rank (owner as from
 * hbi_partition_leaves on hbi_get_leaves' table) */
int hbi_construct_lh_part(hbi_lhp** st_LHp, const hbi_leafmtxp* lf, hbi_ctl* st_ctl, int storage,
                          const int32_t* owner, int rank);

/* HACApK_gen_lattice_vector (m_HACApK_base.f90:3449-3500): ndc = NCELL and
 * lodc(1:ndc) (1-based global ids of the cluster-ordered vector); lodc may be
 * NULL to query ndc only. */
int hbi_gen_lattice_vector(const hbi_ctl* st_ctl, int* ndc, int* lodc);

/* HACApK_adot_lattice_hyp (m_HACApK_solve.f90:220-337): au = H u, host arrays
 * of length ndc in cluster order.  wws (the reference's row scratch) is
 * accepted for signature compatibility and may be NULL. */
int hbi_adot_lattice_hyp(double* au, hbi_lhp* st_LHp, hbi_ctl* st_ctl, double* wws, const double* u);
/* same product on device arrays, enqueued on `stream` (cudaStream_t, NULL =
 * the handle's stream); no synchronisation */
int hbi_adot_lattice_hyp_dev(double* d_au, hbi_lhp* st_LHp, const double* d_u, void* stream);
/* Error check of the asynchronous products (no reference counterpart: the
 * reference's product cannot fail).  Every wait of the product kernels for a
 * bulk copy is bounded (about a second of SM clock); a wait that runs out
 * sets the operator's device error word and the kernel leaves early.  The
 * blocking calls (hbi_adot_lattice_hyp, hbi_rkck, hbi_rkqs, hbi_derivs,
 * hbi_rk_get_state, hbi_cycle_run, hbi_ens_run) read the word themselves and
 * return HBI_ERR_DEVICE; after hbi_adot_lattice_hyp_dev or
 * hbi_adot_lattice_hyp_noalloc, synchronise the stream and call this.
 * Returns HBI_OK or HBI_ERR_DEVICE, and clears the word and the operator's
 * arrival counters, so that the next product starts clean. */
int hbi_lh_check_error(hbi_lhp* st_LHp);
/* Test hook (no reference counterpart): the bound of the product kernels'
 * bulk-copy waits in SM clock cycles for products launched afterwards
 * (operators already bound to an RK handle keep theirs); 0 is a bound that
 * is spent before the first probe, so every wait gives up -- the path of a
 * wait that ran out (error word set, copies in flight drained with the
 * default bound, early exit) without anything being wrong; a negative value
 * restores the default bound.  Ensembles (hbi_ens_create) take the bound of
 * their operators at creation. */
int hbi_lh_set_wait_limit(hbi_lhp* st_LHp, long long cycles);

/* The product of hbi_adot_lattice_hyp_dev without any device allocation.
 * No counterpart in the reference (HACApK allocates its scratch per call).
 * For callers that cannot allocate device memory at the point of the call:
 * a host program whose device memory is owned by another allocator or held
 * under a fixed budget, or a time loop that must not reach cudaMalloc, which
 * can synchronise the whole device.  The per-call scratch (phase-1 sums, the
 * z vectors, the row-group partials and arrival counters) lives in one
 * file-scope device array of HBI_NOALLOC_SCRATCH_BYTES (16 MiB) inside the
 * library, which every GPU that loads the library holds until the process
 * exits.  Operators whose scratch exceeds that return HBI_ERR_LIMIT.  The
 * first call on a device looks up the array's device address (one-time
 * set-up, no allocation); make that first call before any stream capture.
 * All calls share the array and it keeps the previous call's contents (the
 * counters are cleared on every call), so calls that overlap on the GPU --
 * on different streams, or from different threads -- race; serialise them.
 * The array's device address is looked up once per device and kept for the
 * life of the process: do not use this entry point after cudaDeviceReset (or
 * anything else that destroys the device's primary context) in the same
 * process.  Check for a timed-out wait with hbi_lh_check_error. */
#define HBI_NOALLOC_SCRATCH_BYTES (16u << 20)
int hbi_adot_lattice_hyp_noalloc(double* d_au, hbi_lhp* st_LHp, const double* d_u, void* stream);

/* one phase of the product on device arrays: phase 1 forms z = V^T u for the
 * low-rank leaves, phase 2 forms the row groups' partial sums of U z and of
 * the dense leaves (from the z of the last phase 1), phase 3 sums them into
 * au; phase 0 runs all three.  For kernel timing. */
int hbi_adot_lattice_hyp_phase_dev(double* d_au, hbi_lhp* st_LHp, const double* d_u, void* stream, int phase);
/* Launch-shape autotuner of the product kernels (no reference counterpart;
 * it replaces the byte-balanced cut of the leaf list over OpenMP threads,
 * m_HACApK_use.f90:387-431 and m_HACApK_base.f90:1537-1564).  The phase
 * kernels are compiled in several launch shapes (warps per block, stages per
 * warp, stage bytes; the stage size sets the streamed chunk width), each with
 * its own static warp schedule.  hbi_construct_lh times every shape on the
 * new operator (five launches per phase after one warm-up, CUDA events) and
 * keeps the fastest per phase; operators whose plans have the same size
 * statistics reuse the choice; the environment variables HBI_STREAM_SHAPE1=s
 * and HBI_STREAM_SHAPE2=s force shape s of phase 1 / phase 2. */
/* the compiled shapes of phase 1 or 2: *count, and shapes5[5*s .. 5*s+4] =
 * warps per block, stages per warp, stage bytes, variant (phase 1: 0 = the
 * lanes of a column split its rows, 1 = one lane per column; phase 2: how
 * many chunks ahead the multipliers are gathered, minus one), schedule (0 =
 * items over all warps longest first, 1 = per block a run of items
 * consecutive in the store, see hbi_plan_block_schedule, 2 = dynamic: each
 * warp takes the next item from a counter when it needs one, 3 = items dealt
 * over the blocks, each block's warps taking them from a shared counter)
 * (shapes5 may be NULL) */
int hbi_stream_shapes(int phase, int* count, int* shapes5);
/* the shapes chosen for phases 1 and 2, the median time in microseconds of
 * every shape (phase 1's shapes, then phase 2's; -1 if not timed) and how
 * they were chosen (0 timed, 1 reused, 2 forced or pinned) */
int hbi_lh_tuning(const hbi_lhp* st_LHp, int* shape1, int* shape2, float* median_us, int* source);
/* pin the launch shapes of phases 1 and 2 (0 <= shape < count) for products
 * launched afterwards; RK handles copy an operator's shapes when created */
int hbi_lh_set_shapes(hbi_lhp* st_LHp, int shape1, int shape2);
/* Host-only selection rule of the autotuner: times[c * reps + r] are the
 * times of candidate c (non-positive or non-finite entries are ignored);
 * medians[c] receives each candidate's median (-1 when it has no valid
 * time; medians may be NULL); *best is the candidate with the lowest median,
 * a later candidate replacing an earlier one only when it is more than 1%
 * faster.  HBI_ERR_ARG when no candidate has a valid time. */
int hbi_autotune_select(int ncand, int reps, const float* times, float* medians, int* best);
/* algorithmic bytes of phases 1 (V factors + u) and 2 (U factors, dense
 * blocks + u); the product adds ndc x 8 bytes for au (phase 3) */
int hbi_lh_phase_bytes(const hbi_lhp* lh, double* phase1, double* phase2);

/* HACApK_entry_ij (m_HACApK_calc_entry_ij.f90:24-90) evaluated on the GPU for
 * n (i,j) pairs, 1-based global ids. */
int hbi_entry_ij(const hbi_bemv* st_bemv, int n, const int* i, const int* j, double* out);

/* ---- introspection (parity checks, the reference's own export points) ---- */
/* st_ctl%lod(1:nd) after hbi_generate */
int hbi_get_lod(const hbi_ctl* ctl, int* lod);
/* number of leaves and max rank (st_leafmtxp%nlf, %ktmax) */
int hbi_leaf_count(const hbi_leafmtxp* lf, int* nleaf, int* ktmax);
/* leaf table, 6 ints per leaf: ltmtx, kt, nstrtl, ndl, nstrtt, ndt (sorted) */
int hbi_get_leaves(const hbi_leafmtxp* lf, int* leaves6);
/* FP64 factors in the reference's contiguous packing: body offsets
 * (nleaf+1, elements) and the body itself (NULL to query offsets only) */
int hbi_get_body(const hbi_leafmtxp* lf, int64_t* offsets, double* body);
/* algorithmic bytes of one product (factor bytes + vector in/out) */
int hbi_lh_info(const hbi_lhp* lh, int64_t* factor_elems, int64_t* store_bytes, double* alg_bytes);

/* ---- rate-and-state RHS and Cash-Karp RK45 (main_LH.f90:2053-2554) ---- */
typedef struct {
  int ncell;        /* NCELL */
  int evlaw;        /* 0 aging, 1 slip */
  int backslip;     /* matvec input is V - vpl */
  int limitsigma;
  double vref, minsig, maxsig;
  double scale_s, scale_n; /* multipliers of H_s u and H_n u (1/ds0 for 3dph/3dnr) */
  /* per-element parameters in cluster order, length ncell */
  const double *a, *b, *dc, *f0, *taudot, *sigdot, *vpl;
} hbi_rsf_params;

/* binds one (sigma constant) or two H-matrices; lh_n may be NULL */
int hbi_rk_create(hbi_rk** rk, const hbi_rsf_params* p, hbi_lhp* lh_s, hbi_lhp* lh_n);
int hbi_rk_free(hbi_rk* rk);
/* y(3*ncell) interleaved [psi, tau, sigma] per element (main_LH.f90:1208-1215) */
int hbi_rk_set_state(hbi_rk* rk, const double* y);
int hbi_rk_get_state(hbi_rk* rk, double* y);
/* derivs (main_LH.f90:2053-2163): dydx = f(y) */
int hbi_derivs(hbi_rk* rk, const double* y, double* dydx);
/* rkck (main_LH.f90:2472-2554) from the current state; yout/yerr may be NULL */
int hbi_rkck(hbi_rk* rk, double h, double eps, double* yout, double* yerr, double* errmax);
/* rkqs (main_LH.f90:2270-2370): one accepted step from the current state.
 * On success the state advances by *hdid and *x is updated; returns
 * HBI_ERR_CONVERGE when the step size underflows (the reference stops). */
int hbi_rkqs(hbi_rk* rk, double* x, double htry, double eps, double dtmax, double* hdid,
             double* hnext, double* errmax, int* nrjct);
/* after hbi_rk_attempt_async: waits for the handle's stream and returns
 * HBI_ERR_DEVICE if a product kernel gave up a wait (see hbi_lh_check_error) */
int hbi_rk_check_error(hbi_rk* rk);
/* number of kernels the handle launches per RK attempt */
int hbi_rk_launches_per_attempt(const hbi_rk* rk);
/* the CUDA stream (cudaStream_t) the RK handle enqueues on, for timing events */
void* hbi_rk_stream(const hbi_rk* rk);
/* one RK attempt (rkck) enqueued on the handle's stream without any host
 * synchronisation or copy; the error estimate stays on the device */
int hbi_rk_attempt_async(hbi_rk* rk, double h, double eps);

/* ---- time loop on the device (main_LH.f90:1217-1434) ----------------------
 * The reference's loop `do k=kstart,NSTEP`: rkqs, the per-step update of
 * slip and slip rate (:1266-1287), the monitors (:1291-1336), event detection
 * (:1338-1388), field output (:1391-1412) and the stop controls (:1425-1438).
 * Every decision runs on the GPU; the host enqueues attempts ahead of time and
 * drains one small record per attempt (plus field snapshots when the loop
 * writes fields) into the reference's output files:
 *   monitor<number>.dat, time<number>.dat, event<number>.dat (text) and
 *   vel/slip/sigma/tau/EQslip<number>.dat (stream binary, cluster order). */
typedef struct hbi_cycle_s hbi_cycle;
typedef struct {
  double eps_r;        /* RK tolerance */
  double dtinit;       /* first trial step (s) */
  double dtmax;        /* s */
  double tmax;         /* s (the reference converts its years at :330) */
  double velth, velmax, velmin;
  double dtout_inter;  /* s */
  double dtout_co;     /* s */
  double rigid;        /* rigidity of the event magnitude (m_const.f90) */
  long long nstep;     /* NSTEP */
  long long interval;  /* field output every `interval` steps; 0 = NSTEP */
  int number;          /* output file number */
  int inflight;        /* attempts enqueued ahead of the host, 1..16 */
  int pad0, pad1;
  const char* outdir;  /* directory for the output files; NULL = no files */
} hbi_cycle_params;

#define HBI_STOP_NONE 0
#define HBI_STOP_TMAX 1      /* x > tmax */
#define HBI_STOP_VELMAX 2    /* max slip rate > velmax */
#define HBI_STOP_VELMIN 3    /* max slip rate < velmin */
#define HBI_STOP_KLIMIT 4    /* k reached the run's step limit (resumable) */
#define HBI_STOP_UNDERFLOW 5 /* rkqs step size underflow (reference: stop) */
#define HBI_STOP_TLIMIT 6    /* x reached the run's time limit exactly (resumable) */
#define HBI_STOP_DEVICE 7    /* a product kernel gave up a wait; hbi_cycle_run returns HBI_ERR_DEVICE */

typedef struct {
  long long k, attempts, rejected;
  double x, hnext, errmax, dtdid;
  double mvel, meanslip, meanmu, maxnorm, minnorm;
  int nrjct, events, slipping, stop;
  double wall_s;       /* host wall time of the run call */
} hbi_cycle_status;

typedef struct {
  int id, hypoloc;     /* event number; 1-based cluster-order index of max slip rate at onset */
  long long k;         /* step at which the event ended */
  double onset, end;   /* s */
  double moment;       /* mean slip of the event (m) */
  double mw;           /* (log10(moment*rigid*sg)+5.9)/1.5 as event*.dat */
} hbi_event;

/* Starts a loop from the RK handle's current state (hbi_rk_set_state), with
 * slip rate vel (ncell, cluster order: the reference's `vel` before the loop)
 * and element areas ds (ncell, cluster order: ds(lodc(i))).  Writes the k=0
 * outputs.  The RK handle must outlive the loop. */
int hbi_cycle_create(hbi_cycle** c, hbi_rk* rk, const double* vel, const double* ds, const hbi_cycle_params* p);
/* Runs until a stop control fires, until k reaches k_limit (<=0: none) or x
 * reaches t_limit (<=0: none; the last step is shortened to land on it). */
int hbi_cycle_run(hbi_cycle* c, long long k_limit, double t_limit, hbi_cycle_status* st);
/* Restart (main_LH.f90:836-957): continue the loop of an earlier run with the
 * same outdir, number and interval.  From monitor<number>.dat the last step k
 * that is a multiple of `interval` gives x and the next trial step
 * min(2 dtdid, 0.9 dtdid errmax^-0.2); the last snapshots of the vel, slip,
 * sigma and tau files give the state (psi from vel, tau, sigma, main_LH.f90:
 * 899).  The loop resumes at step k + 1, appends to the files (EQslip starts
 * anew) and does not rewrite monitor lines already in the file. */
int hbi_cycle_restart(hbi_cycle** c, hbi_rk* rk, const double* ds, const hbi_cycle_params* p);
/* the restart point of a monitor file: k, x, next trial step, last step listed */
int hbi_restart_point(const char* monitor_path, long long interval, long long* k, double* x, double* dtnxt,
                      long long* kend);
/* slip and slip rate (ncell, cluster order); the state y via hbi_rk_get_state */
int hbi_cycle_fields(hbi_cycle* c, double* vel, double* slip);
/* finished events so far; *count = their number (up to max are copied) */
int hbi_cycle_events(hbi_cycle* c, hbi_event* ev, int max, int* count);
/* per attempt: k, x, h, errmax, accepted, mvel, hnext, nrjct (8 doubles each) */
int hbi_cycle_trace(hbi_cycle* c, double* rec, long long max, long long* count);
int hbi_cycle_free(hbi_cycle* c);
/* Learned step-size proposer (no reference counterpart).  After each accepted
 * step an MLP (nin -> hid -> hid -> 1, tanh) maps the loop's history to
 * d = log10(h_next / rkqs h_next), clamped to [lo, hi]; the next attempt uses
 * rkqs's h_next * 10^d.  The rkqs error test still judges every attempt and
 * its shrink rule still handles every rejection.  w (floats, layout
 * W1[hid][nin] b1 W2[hid][hid] b2 W3[hid] b3 mean[nin] sd[nin] lo hi) is
 * copied; NULL turns the proposer off. */
int hbi_cycle_set_proposer(hbi_cycle* c, const float* w);
int hbi_cycle_proposer_size(int* nin, int* hid, int* nfloats);

/* ---- training of the step-size proposer (no reference counterpart) -------
 * An MLP nin -> hid -> hid -> 1 (tanh, tanh, linear) trained by mean squared
 * error with Adam, entirely by this library's kernels (forward, backward,
 * update).  Parameters are packed W1[hid][nin] b1 W2[hid][hid] b2 W3[hid] b3,
 * the first part of the proposer's weight vector. */
typedef struct hbi_mlp_s hbi_mlp;
int hbi_mlp_create(hbi_mlp** m, int nin, int hid, int batch_max);
int hbi_mlp_free(hbi_mlp* m);
int hbi_mlp_set_params(hbi_mlp* m, const float* p);
int hbi_mlp_get_params(hbi_mlp* m, float* p);
/* the training loss: tau <= 0 the squared error (the default), 0 < tau < 1
 * the pinball loss of quantile tau -- (1 - tau) r for r = out - t > 0, -tau r
 * otherwise -- whose minimiser is the tau-quantile of t given the inputs */
int hbi_mlp_set_loss(hbi_mlp* m, float tau);
/* loss = mean of the per-sample loss over x[batch][nin]; grad = d loss / d params */
int hbi_mlp_loss_grad(hbi_mlp* m, const float* x, const float* t, int batch, float* grad, float* loss,
                      float* out);
/* `epochs` passes of Adam over n samples in shuffled minibatches (seeded) */
int hbi_mlp_train(hbi_mlp* m, const float* x, const float* t, long long n, int epochs, int batch, float lr,
                  unsigned long long seed, float* loss_per_epoch);
int hbi_mlp_predict(hbi_mlp* m, const float* x, long long n, float* out);

/* Host-only self check of the product's work plan (no GPU, no reference
 * counterpart): builds the row-tiled stores and work items for a leaf list
 * leaves6[nleaf][6] = {ltmtx, kt, nstrtl, ndl, nstrtt, ndt} with vec elements
 * per 16 bytes, checks every bound the kernels rely on, and evaluates y = H x
 * from the HACApK-packed FP64 body by walking the items as the kernels do.
 * stats[8]: items of phase 1 and 2, V and U store elements, z length,
 * phase-1 and phase-2 partials, conversion segments.  HBI_ERR_STATE names the
 * violated bound. */
int hbi_plan_emulate(int n, int nleaf, const int* leaves6, const double* body, int vec, const double* x,
                     double* y, int64_t* stats);
/* Host-only (no reference counterpart): the static warp schedule the product
 * kernels walk -- n items of the given costs dealt longest-first to the
 * least-loaded of nwarps warps.  woff[nwarps + 1] and witem[n] receive the
 * CSR lists (warp w: witem[woff[w] .. woff[w+1])). */
int hbi_plan_warp_schedule(int n, const int64_t* cost, int nwarps, int32_t* woff, int32_t* witem);
/* Host-only (no reference counterpart): the schedule with locality -- the n
 * items in order of key (their store offset) cut into nblocks consecutive
 * runs of near-equal cost, each run dealt longest-first over its block's nw
 * warps; woff[nblocks * nw + 1], witem[n] as hbi_plan_warp_schedule (warp
 * b * nw + w). */
int hbi_plan_block_schedule(int n, const int64_t* cost, const int64_t* key, int nblocks, int nw, int32_t* woff,
                            int32_t* witem);

/* ---- ensemble of simulations sharing one H-matrix pair (no reference
 * counterpart; configuration c4) -----------------------------------------
 * `members` rate-and-state systems with per-member friction parameters b
 * and dc run on the same lh_s / lh_n: every RK stage applies each H-matrix to
 * all members' slip rates at once (a multi-vector product), and each member
 * keeps its own FP64 state, step size and rkqs controller (main_LH.f90:
 * 2270-2370).  Arrays are cluster order with the member index fastest:
 * y[(3*i + c) * members + m], b[i * members + m].  p supplies a, f0, taudot,
 * sigdot, vpl (per element) and the law; its b and dc are ignored. */
typedef struct hbi_ens_s hbi_ens;
typedef struct {
  long long attempts;   /* ensemble attempts (each advances every active member) */
  long long steps;      /* accepted member steps, summed over members */
  long long rejected;   /* rejected member attempts, summed */
  int done, failed;     /* members that reached t_limit; members whose step size underflowed */
  double wall_s;
} hbi_ens_status;
int hbi_ens_create(hbi_ens** e, const hbi_rsf_params* p, hbi_lhp* lh_s, hbi_lhp* lh_n, int members,
                   const double* b, const double* dc);
int hbi_ens_free(hbi_ens* e);
/* y (3*ncell*members), vel (ncell*members: the slip rate before the loop) */
int hbi_ens_set_state(hbi_ens* e, const double* y, const double* vel);
int hbi_ens_get_state(hbi_ens* e, double* y, double* slip, double* x);
/* Run the ensemble's multi-vector product on the tensor cores (tcgen05,
 * BF16 hi + lo operands, FP32 accumulation in tensor memory) built from the
 * FP64 factors of the generate calls lh_s / lh_n were made from. */
int hbi_ens_use_tensor_cores(hbi_ens* e, const hbi_leafmtxp* lf_s, const hbi_leafmtxp* lf_n);
/* every member from x = 0 to exactly t_limit (s) */
int hbi_ens_run(hbi_ens* e, double eps_r, double dtinit, double dtmax, double t_limit, hbi_ens_status* st);
/* One multi-vector product of both H-matrices (the kernels the run uses:
 * tensor cores after hbi_ens_use_tensor_cores, else CUDA cores) applied to the
 * 64 members' vectors x[i * 64 + m] (cluster order, FP32, host): ys = H_s x,
 * yn = H_n x (yn unused with one matrix), same layout.  With reps > 0 the
 * product (phase 1, phase 2, group sums) is repeated reps more times and *ms
 * receives the CUDA-event time of one.  Overwrites the ensemble's product
 * input buffer (the next attempt rewrites it from the state).  The
 * counterpart of HACApK_adot_lattice_hyp (m_HACApK_solve.f90:220) for 64
 * right-hand sides. */
int hbi_ens_product(hbi_ens* e, const float* x, float* ys, float* yn, int reps, double* ms);

/* Host-only self check of the tensor-core plan of the ensemble product (no
 * reference counterpart): y = H x through that plan with the factors rounded
 * to BF16 hi + lo as stored, and every bound its kernels rely on.
 * stats[4]: items of phase 1 and 2, store elements of phase 1 and 2. */
int hbi_tc_plan_emulate(int n, int nleaf, const int* leaves6, const double* body, const double* x, double* y,
                        int64_t* stats);

/* Self test of the tensor-core path (no reference counterpart): one
 * tcgen05 MMA, D[128][64] = A[128][16] * B[64][16]^T with BF16 operands (raw
 * bit patterns) from canonical K-major shared-memory layouts and FP32
 * accumulation in tensor memory.  variant 0 uses the descriptor convention of
 * the ensemble kernels; variant 1 swaps its two stride fields; variant 2 is an
 * M = 64 MMA (rows 0-63 of a), d holding all 128 tensor-memory lanes. */
int hbi_umma_probe(const uint16_t* a, const uint16_t* b, float* d, int variant);

#ifdef __cplusplus
}
#endif
#endif
