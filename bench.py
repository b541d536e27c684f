#!/usr/bin/env python
"""bench.py -- H-matvec GB/s inside Cash-Karp RK45 attempts of HBI's hot path,
and the simulated years per hour of the time loop on the target fault.

Kernel workload (the headline `value`): the 3D planar thrust fault of the
second benchmark configuration -- a 30-degree dipping fault in a half space,
Okada kernel, 256 x 256 = 65,536 elements, two H-matrices (shear 's' and
normal 'n'), velocity-weakening central patch, ACA eps 1e-5; seeded
synthetic inputs.  A step is one Cash-Karp attempt (rkck, main_LH.f90:
2472-2554): six stages, each evaluating derivs (main_LH.f90:2053-2163) with
one product per H-matrix, i.e. 12 lattice H-matrix-vector products plus the
fused rate-and-state / stage epilogue.  value = 12 x (algorithmic bytes of
one product) per second, the bytes being the stored factor bytes
(sum_LR kt(ndl+ndt) + sum_dense ndl*ndt, times the storage size) plus the
FP64 input and output vectors.  The factor stores (> 1 GB) exceed the 126 MB
L2, so no flush is needed between steps.  The same attempt rate with FP64
factors, the reference's own precision, is reported beside it
(same_precision_f64).

Time-loop workload (sim_yr_per_hour): the third configuration, the target of
the 3x goal -- a rough strike-slip fault of 200,000 triangles, TDstressFS
full space, slip law, two H-matrices, ACA eps 1e-4 -- from steady state
through its first earthquake (it nucleates at 19.44 years) to
--sim-window-yr (20): the plain form (FP64 factors, rkqs controller) against
the mixed form (FP32 factors and the learned step-size proposer trained on
the plain run's trace), with the catalogues compared event by event (see
catalogue_gate) and the slip field at the window's end, each within 1e-3
relative; a mismatch fails the gate and is listed, never dropped.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--store f32|bf16|f64]
  python bench.py --impl reference ...   # the CPU oracle port, all host cores
  python bench.py --mode matvec|ensemble  # product kernels alone / configuration c4
  python bench.py --mode kernels --imax 128 --jmax 128  # one small run of every other kernel (for ncu)
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NSMI_Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
          "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
          "clocks_event_reasons.sw_power_cap")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--store", default="f32", choices=["f64", "f32", "bf16"])
    ap.add_argument("--imax", type=int, default=256)
    ap.add_argument("--jmax", type=int, default=256)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-same-precision", action="store_true")
    ap.add_argument("--mode", default="step", choices=["step", "matvec", "ensemble", "kernels"])
    ap.add_argument("--sim-config", default="c3", choices=["c3", "c2"],
                    help="workload of the sim-yr/h comparison (c3: the 200,000-triangle rough fault)")
    ap.add_argument("--sim-window-yr", type=float, default=20.0,
                    help="simulated window of the sim-yr/h comparison (0: skip it)")
    ap.add_argument("--window-yr", type=float, default=2.0, help="simulated window of --mode ensemble")
    return ap.parse_args()


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index):
        self.index = index
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={NSMI_Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except FileNotFoundError:
            self.p = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            self.p.wait()

    def summary(self):
        self.f.flush()
        rows = [l.split(",") for l in open(self.f.name).read().splitlines() if l.strip()]
        os.unlink(self.f.name)
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx = max(mx, float(r[2]))
                for k, nm in enumerate(names):
                    if r[5 + k].strip().lower() == "active":
                        reasons.add(nm)
            except (ValueError, IndexError):
                pass
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


# DRAM bytes (read + write) per launch of the phase kernels on the c2 shear
# H-matrix, from the ncu captures summarised under profiles/ (one entry per
# factor storage that has been captured)
NCU_TRAFFIC = {
    "f32": {"phase1": 327.2e6, "phase2": 376.6e6, "source": "profiles/matvec_p1_p2_c2_256x256_f32.md"},
    "f64": {"phase1": 651.7e6, "phase2": 738.5e6, "source": "profiles/matvec_p1_p2_c2_256x256_f32.md (FP64 lines)"},
}


def dist_init():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def workload(args):
    from hbi_gb300 import configs
    return configs.c2_3dph(args.imax, args.jmax)


def out_line(d):
    print(json.dumps(d), flush=True)


def time_phases(torch, lh, n, reps):
    """Mean device time of the three product phases, timed with CUDA events
    on the (non-default) stream they are launched on."""
    x = torch.randn(n, dtype=torch.float64, device="cuda")
    y = torch.empty(n, dtype=torch.float64, device="cuda")
    ts = torch.cuda.Stream()
    for _ in range(3):
        lh.matvec_dev(y.data_ptr(), x.data_ptr(), ts.cuda_stream)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4 * reps)]
    torch.cuda.synchronize()
    for r in range(reps):
        ev[4 * r].record(ts)
        lh.matvec_dev(y.data_ptr(), x.data_ptr(), ts.cuda_stream, phase=1)
        ev[4 * r + 1].record(ts)
        lh.matvec_dev(y.data_ptr(), x.data_ptr(), ts.cuda_stream, phase=2)
        ev[4 * r + 2].record(ts)
        lh.matvec_dev(y.data_ptr(), x.data_ptr(), ts.cuda_stream, phase=3)
        ev[4 * r + 3].record(ts)
    torch.cuda.synchronize()
    lh.check_error()
    t1 = float(np.mean([ev[4 * r].elapsed_time(ev[4 * r + 1]) for r in range(reps)])) * 1e-3
    t2 = float(np.mean([ev[4 * r + 1].elapsed_time(ev[4 * r + 2]) for r in range(reps)])) * 1e-3
    t3 = float(np.mean([ev[4 * r + 2].elapsed_time(ev[4 * r + 3]) for r in range(reps)])) * 1e-3
    b1, b2 = lh.phase_bytes()
    return t1, t2, t3, b1, b2


def run_matvec_mode(args):
    """Products only (no RK, no CPU baseline): the target of kernel profiles."""
    import torch

    import hbi_gb300 as H
    w = workload(args)
    n = w.nd
    ctl = H.Ctl(n)
    lf = H.LeafMtxp(ctl, w.geometry("s"), w.eps_h)
    lh = H.LHp(lf, ctl, args.store)
    t1, t2, t3, b1, b2 = time_phases(torch, lh, n, args.steps)
    out_line({"mode": "matvec", "elements": n, "storage": args.store, "phase1_us": round(t1 * 1e6, 2),
              "phase2_us": round(t2 * 1e6, 2), "phase3_us": round(t3 * 1e6, 2), "phase1_gbs": round(b1 / t1 / 1e9, 1),
              "phase2_gbs": round(b2 / t2 / 1e9, 1),
              "product_gbs": round((b1 + b2 + 8 * n) / (t1 + t2 + t3) / 1e9, 1), "bytes": b1 + b2 + 8 * n})


def run_ensemble_mode(args):
    """Configuration c4: 64 simulations with their own b and dc sharing the c2
    H-matrices (FP32), every member from steady state to --window-yr; against
    one member run alone through the single-system loop on the same window."""
    import hbi_gb300 as H
    from hbi_gb300 import configs
    w = workload(args)
    n = w.nd
    ctl_s, ctl_n = H.Ctl(n), H.Ctl(n)
    lf_s = H.LeafMtxp(ctl_s, w.geometry("s"), w.eps_h)
    lf_n = H.LeafMtxp(ctl_n, w.geometry("n"), w.eps_h)
    lh_s, lh_n = H.LHp(lf_s, ctl_s, "f32"), H.LHp(lf_n, ctl_n, "f32")
    ndc, lodc = H.HACApK_gen_lattice_vector(ctl_s)
    b_in, dc_m = configs.ensemble_params(64, seed=0)
    y, vel, b, dc, p = configs.ensemble_state(w, lodc, b_in, dc_m)
    T = args.window_yr * H.YEAR
    res, prod_ms = {}, {}
    # algorithmic bytes of one multi-vector product: both factor stores once,
    # the 64 members' input vectors, both outputs
    prod_bytes = lh_s.info()["store_bytes"] + lh_n.info()["store_bytes"] + 3 * n * 64 * 4
    X = np.random.default_rng(0).standard_normal((n, 64)).astype(np.float32)
    for product in ("cuda-cores", "tcgen05"):
        ens = H.Ensemble(lh_s, lh_n, b, dc, evlaw=w.evlaw, scale=w.scale, a=p["a"], f0=p["f0"], vpl=p["vpl"])
        if product == "tcgen05":
            ens.use_tensor_cores(lf_s, lf_n)
        ens.product(X, reps=3)
        prod_ms[product] = ens.product(X, reps=20)[2]
        ens.set_state(y, vel)
        st = ens.run(T, eps_r=1e-6)
        ye, se, xe = ens.get_state()
        res[product] = (st, ye)
        ens.close()
    st, ye = res["tcgen05"]
    ds = w.ds_area[lodc - 1]
    m = 0
    rk = H.RK(lh_s, lh_n, evlaw=w.evlaw, scale=w.scale, a=p["a"], b=b[:, m], dc=dc[:, m], f0=p["f0"], vpl=p["vpl"])
    rk.set_state(y[:, m])
    cyc = H.Cycle(rk, vel[:, m], ds, eps_r=1e-6)
    cs = cyc.run(t_limit=T)
    y1 = rk.get_state()
    member_yr_h = 64 * args.window_yr / st["wall_s"] * 3600
    single_yr_h = args.window_yr / cs["wall_s"] * 3600
    out_line({"mode": "ensemble", "workload": f"c4: 64 members on {w.name}", "members": 64,
              "window_yr": args.window_yr, "wall_s": round(st["wall_s"], 2), "attempts": st["attempts"],
              "member_steps": st["steps"], "member_rejected": st["rejected"], "done": st["done"],
              "ms_per_attempt": round(st["wall_s"] / max(1, st["attempts"]) * 1e3, 3),
              "member_sim_yr_per_hour": round(member_yr_h, 1),
              "single_sim_yr_per_hour": round(single_yr_h, 1), "throughput_ratio": round(member_yr_h / single_yr_h, 2),
              "member0_state_rel_diff": float(np.linalg.norm(ye[:, 0] - y1) / np.linalg.norm(y1)),
              "product": "tcgen05 (BF16 hi+lo, FP32 accumulation in tensor memory)",
              "cuda_core_product_ms_per_attempt": round(res["cuda-cores"][0]["wall_s"] /
                                                        max(1, res["cuda-cores"][0]["attempts"]) * 1e3, 3),
              "product_ms": {k: round(v, 4) for k, v in prod_ms.items()},
              "product_gbs": {k: round(prod_bytes / (v * 1e-3) / 1e9, 1) for k, v in prod_ms.items()},
              "product_bytes": prod_bytes,
              "product_frac_of_hbm": {k: round(prod_bytes / (v * 1e-3) / 1e9 / peaks()[0], 3)
                                      for k, v in prod_ms.items()}})


# ------------------------------------------------------------ time loops
def compare_time_loops(args, w):
    """sim-yr/h of the time loop over [0, window]: the plain FP64 form (FP64
    factors, rkqs controller) against the mixed form (--store factors,
    learned step-size proposer trained on the plain run's own trace)."""
    import hbi_gb300 as H
    from hbi_gb300 import proposer
    from hbi_gb300.catalogue import catalogue_gate
    n = w.nd
    t0 = time.perf_counter()
    ctl_s, ctl_n = H.Ctl(n), H.Ctl(n)
    lf_s = H.LeafMtxp(ctl_s, w.geometry("s"), w.eps_h)
    lf_n = H.LeafMtxp(ctl_n, w.geometry("n"), w.eps_h)
    t_gen = time.perf_counter() - t0
    ndc, lodc = H.HACApK_gen_lattice_vector(ctl_s)
    y0, p = w.initial_state(lodc)
    ds = w.ds_area[lodc - 1]
    T = args.sim_window_yr * H.YEAR

    def one(store, wts=None):
        lh_s = H.LHp(lf_s, ctl_s, store)
        lh_n = H.LHp(lf_n, ctl_n, store)
        gb = (lh_s.info()["store_bytes"] + lh_n.info()["store_bytes"]) / 1e9
        rk = H.RK(lh_s, lh_n, evlaw=w.evlaw, scale=w.scale, a=p["a"], b=p["b"], dc=p["dc"], f0=p["f0"],
                  vpl=p["vpl"])
        rk.set_state(y0)
        c = H.Cycle(rk, p["vel"], ds, eps_r=1e-6, tmax_yr=max(w.tmax_yr, args.sim_window_yr + 1))
        if wts is not None:
            c.set_proposer(wts)
        st = c.run(t_limit=T)
        out = dict(st=st, trace=c.trace(), events=c.events(), slip=c.fields()[1], store_gb=gb)
        c.close()
        rk.close()
        lh_s.close()
        lh_n.close()
        return out

    plain = one("f64")
    X, Tt = proposer.training_set(plain["trace"])
    t1 = time.perf_counter()
    wts, hist = proposer.train(X, Tt, epochs=30)
    t_train = time.perf_counter() - t1
    mixed = one(args.store, wts)
    for h in (lf_s, lf_n, ctl_s, ctl_n):
        h.close()
    rate = lambda r: r["st"]["x"] / H.YEAR / r["st"]["wall_s"] * 3600.0
    rj = lambda r: r["st"]["rejected"] / max(1, r["st"]["attempts"])
    cat = lambda r: [[round(e["onset"] / H.YEAR, 6), round(e["end"] / H.YEAR, 6), e["hypoloc"],
                      float("%.6e" % e["moment"])] for e in r["events"]]
    return {
        "unit": "simulated yr/hour", "workload": f"{w.name}: {n} elements, 2 H-matrices, ACA eps {w.eps_h}, "
                                                 f"eps_r 1e-6, from steady state to {args.sim_window_yr} yr",
        "window_yr": args.sim_window_yr,
        "plain_fp64": round(rate(plain), 2), "mixed": round(rate(mixed), 2),
        "ratio": round(rate(mixed) / rate(plain), 3),
        "mixed_form": f"{args.store} factors ({mixed['store_gb']:.1f} GB) + learned step-size proposer (trained on "
                      f"the plain run's trace, {len(Tt)} samples, {t_train:.1f} s on the GPU)",
        "plain_form": f"f64 factors ({plain['store_gb']:.1f} GB), rkqs controller, same kernels and "
                      f"device-resident loop",
        "gate": catalogue_gate(plain, mixed),
        "events": [len(plain["events"]), len(mixed["events"])],
        "catalogue_plain": cat(plain), "catalogue_mixed": cat(mixed),
        "attempts": [plain["st"]["attempts"], mixed["st"]["attempts"]],
        "rejected_frac": [round(rj(plain), 4), round(rj(mixed), 4)],
        "ms_per_attempt": [round(r["st"]["wall_s"] / max(1, r["st"]["attempts"]) * 1e3, 3) for r in (plain, mixed)],
        "wall_s": [round(plain["st"]["wall_s"], 2), round(mixed["st"]["wall_s"], 2)],
        "assembly_s": round(t_gen, 1),
    }


# --------------------------------------------------------------------- ours
def attempt_rate(torch, rk, steps, warmup, world, local, dist=None, clocks=False):
    """K back-to-back RK attempts enqueued on the handle's stream, timed with
    CUDA events on that stream; max over ranks."""
    stream = torch.cuda.ExternalStream(rk.stream)
    h, eps = 1.0e5, 1e-5
    for _ in range(warmup):
        rk.attempt_async(h, eps)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ck = Clocks(local) if clocks else None
    if ck:
        ck.__enter__()
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(steps):
        rk.attempt_async(h, eps)
    e1.record(stream)
    torch.cuda.synchronize()
    if ck:
        ck.__exit__()
    rk.check_error()
    ms = e0.elapsed_time(e1)
    if world > 1:
        tt = torch.tensor([ms], device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        ms = float(tt.item())
    return ms, (ck.summary() if ck else None)


def e2e_rate(torch, rk, y0, steps, world, dist=None):
    """The same attempts through the C ABI with pinned host buffers: state
    copied in, rkck, yout and yerr copied out, every step."""
    n3 = y0.size
    yh = torch.empty(n3, dtype=torch.float64, pin_memory=True).numpy()
    yh[:] = y0
    yo = torch.empty(n3, dtype=torch.float64, pin_memory=True).numpy()
    ye = torch.empty(n3, dtype=torch.float64, pin_memory=True).numpy()
    h, eps = 1.0e5, 1e-5
    for _ in range(2):
        rk.set_state(yh)
        rk.rkck_into(h, eps, yo, ye)
    torch.cuda.synchronize()
    te = time.perf_counter()
    for _ in range(steps):
        rk.set_state(yh)
        rk.rkck_into(h, eps, yo, ye)
    te = time.perf_counter() - te
    if world > 1:
        tt = torch.tensor([te], device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        te = float(tt.item())
    return te, {"h2d_bytes_per_step": n3 * 8, "d2h_bytes_per_step": 2 * n3 * 8 + 32}


def run_ours(args):
    import torch

    import hbi_gb300 as H

    rank, world, local = dist_init()
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    H.set_device(local)
    w = workload(args)
    n = w.nd
    t0 = time.perf_counter()
    ctl_s, ctl_n = H.Ctl(n), H.Ctl(n)
    lf_s = H.LeafMtxp(ctl_s, w.geometry("s"), w.eps_h)
    lf_n = H.LeafMtxp(ctl_n, w.geometry("n"), w.eps_h)
    t_gen = time.perf_counter() - t0
    ndc, lodc = H.HACApK_gen_lattice_vector(ctl_s)
    y0, p = w.initial_state(lodc)

    def rk_for(store):
        lh_s = H.LHp(lf_s, ctl_s, store)
        lh_n = H.LHp(lf_n, ctl_n, store)
        rk = H.RK(lh_s, lh_n, evlaw=w.evlaw, scale=w.scale, a=p["a"], b=p["b"], dc=p["dc"], f0=p["f0"],
                  vpl=p["vpl"], taudot=p["taudot"], sigdot=p["sigdot"])
        rk.set_state(y0)
        bytes_attempt = 6.0 * (lh_s.info()["alg_bytes"] + lh_n.info()["alg_bytes"])
        return rk, lh_s, lh_n, bytes_attempt

    # ---- the headline store: device-resident attempts, roofline, end to end ----
    rk, lh_s, lh_n, bytes_attempt = rk_for(args.store)
    t_setup = time.perf_counter() - t0
    info_s, info_n = lh_s.info(), lh_n.info()
    ms, clocks = attempt_rate(torch, rk, args.steps, args.warmup, world, local, dist, clocks=True)
    ms_step = ms / args.steps
    value = world * args.steps * bytes_attempt / (ms * 1e-3) / 1e9
    t1, t2, t3, b1, b2 = time_phases(torch, lh_s, n, 20)
    peak, peak_kind = peaks()
    dominant = "phase2" if t2 >= t1 else "phase1"
    ach = (b2 / t2 if dominant == "phase2" else b1 / t1) / 1e9
    mv_gbs = (b1 + b2 + 8 * n) / (t1 + t2 + t3) / 1e9  # the whole product (y written by phase 3)
    te, e2e_bytes = e2e_rate(torch, rk, y0, args.steps, world, dist)
    e2e = world * args.steps * bytes_attempt / te / 1e9
    launches = args.steps * rk.launches_per_attempt
    for hnd in (rk, lh_s, lh_n):
        hnd.close()

    # ---- the same attempts with FP64 factors (the reference's precision) ----
    same = None
    if args.store != "f64" and not args.no_same_precision:
        rk, lh_s, lh_n, bytes64 = rk_for("f64")
        ms64, _ = attempt_rate(torch, rk, args.steps, args.warmup, world, local, dist)
        te64, _ = e2e_rate(torch, rk, y0, args.steps, world, dist)
        same = {"storage": "f64", "value": round(world * args.steps * bytes64 / (ms64 * 1e-3) / 1e9, 2),
                "unit": "GB/s", "ms_per_step": round(ms64 / args.steps, 4),
                "e2e": {"value": round(world * args.steps * bytes64 / te64 / 1e9, 2), "unit": "GB/s",
                        "ms_per_step": round(te64 / args.steps * 1e3, 4)},
                "note": "same attempts, FP64 factor stores: FP64 products with FP64 accumulation"}
        for hnd in (rk, lh_s, lh_n):
            hnd.close()

    # ---- CPU baseline: the oracle port on the host cores (rank 0, N=1) ----
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(args, w, lf_s, lf_n, y0, p)
    for hnd in (lf_s, lf_n, ctl_s, ctl_n):
        hnd.close()

    # ---- sim-yr/h: plain FP64 form against the mixed + learned form (one
    # GPU runs only: the comparison takes minutes, and the other ranks of a
    # multi-GPU run would hold their GPUs idle meanwhile) ----
    cyc = None
    if rank == 0 and world == 1 and args.sim_window_yr > 0:
        from hbi_gb300 import configs
        cyc = compare_time_loops(args, configs.c3_3dnt() if args.sim_config == "c3" else w)

    if rank == 0:
        traffic = NCU_TRAFFIC.get(args.store, {})
        d = {
            "metric": "H-matvec GB/s", "value": round(value, 2), "unit": "GB/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_step, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": args.store,
            "data": "synthetic (seeded 3D planar thrust, Okada half space; seeded rough fault for sim_yr_per_hour)",
            "config": {"workload": f"{w.name}: 3dph Okada half space, {n} elements, 2 H-matrices (s,n), "
                                   f"ACA eps {w.eps_h}, one Cash-Karp attempt per step (12 products)",
                       "elements": n, "storage": args.store, "products_per_step": 12,
                       "l2": "inputs larger than L2 (factor stores %.2f GB)" % (
                           (info_s["store_bytes"] + info_n["store_bytes"]) / 1e9),
                       "parallelism": f"replicas x{world}" if world > 1 else "1 GPU"},
            "roofline": {"bound": "hbm", "kernel": f"matvec {dominant}", "achieved": round(ach, 1),
                         "peak": peak, "unit": "GB/s", "frac": round(ach / peak, 4), "peak_kind": peak_kind,
                         "traffic": traffic.get(dominant), "traffic_source": traffic.get("source"),
                         "matvec_gbs_whole_product": round(mv_gbs, 1),
                         "phase1_us": round(t1 * 1e6, 2), "phase2_us": round(t2 * 1e6, 2),
                         "phase3_us": round(t3 * 1e6, 2),
                         "phase1_bytes": b1, "phase2_bytes": b2},
            "e2e": dict({"value": round(e2e, 2), "unit": "GB/s"}, **e2e_bytes),
            "gpu_launches": launches,
            "clocks": clocks,
            "setup": {"generate_s": round(t_gen, 2), "total_s": round(t_setup, 2),
                      "factor_elems_s": info_s["factor_elems"], "factor_elems_n": info_n["factor_elems"],
                      "compression_s": info_s["factor_elems"] / n / n},
        }
        if same:
            d["same_precision_f64"] = same
        if cpu:
            d["cpu_baseline"] = cpu
        if cyc:
            d["sim_yr_per_hour"] = cyc
        out_line(d)
    if world > 1:
        dist.destroy_process_group()


def cpu_baseline(args, w, lf_s, lf_n, y0, p):
    """The oracle's RK attempt (OpenMP products mirroring the reference's
    thread ranges and atomics) on the same FP64 factors, all host cores."""
    from oracle import oracle as O
    O.build()
    n = w.nd
    off, body = lf_s.body()
    Hs = O.HMatrix.from_body(n, lf_s.leaves(), off, body)
    off, body = lf_n.body()
    Hn = O.HMatrix.from_body(n, lf_n.leaves(), off, body)
    cores = os.cpu_count() or 1
    R = O.RSF(n, Hs, Hn, evlaw=w.evlaw, divide_ds0=1, ds0=w.w, nthreads=cores, a=p["a"], b=p["b"], dc=p["dc"],
              f0=p["f0"], vplv=p["vpl"], taudot=p["taudot"], sigdot=p["sigdot"])
    R.rkck(y0, 0.0, 1e5)
    t = time.perf_counter()
    k = 0
    while True:
        R.rkck(y0, 0.0, 1e5)
        k += 1
        if time.perf_counter() - t > args.cpu_seconds or k >= 200:
            break
    t = time.perf_counter() - t
    bytes_attempt = 6.0 * ((Hs.body.size + Hn.body.size) * 8 + 2 * 2 * n * 8)
    return {"value": round(k * bytes_attempt / t / 1e9, 3), "unit": "GB/s", "cores": cores, "kind": "port",
            "sample": f"{k} Cash-Karp attempts of the same workload on the same FP64 factors "
                      f"({(Hs.body.size + Hn.body.size) * 8 / 1e9:.2f} GB), oracle rkck with OpenMP products",
            "ms_per_step": round(t / k * 1e3, 2)}


# ---------------------------------------------------------------- reference
def run_reference(args):
    rank, world, local = dist_init()
    if rank != 0:
        return
    from oracle import oracle as O
    O.build()
    w = workload(args)
    n = w.nd
    cores = os.cpu_count() or 1
    coord = np.stack([w.geom_kw["xcol"], w.geom_kw["ycol"], w.geom_kw["zcol"]], 1)
    t0 = time.perf_counter()
    lod, lv, _ = O.build_structure(coord)
    p = O.default_params()
    p[70] = w.eps_h
    Hs = O.HMatrix(O.Geometry(2, n, "s", w=w.w, **w.geom_kw), lod, lv, p, nthreads=cores)
    Hn = O.HMatrix(O.Geometry(2, n, "n", w=w.w, **w.geom_kw), lod, lv, p, nthreads=cores)
    t_setup = time.perf_counter() - t0
    y0, pp = w.initial_state(lod)
    R = O.RSF(n, Hs, Hn, evlaw=w.evlaw, divide_ds0=1, ds0=w.w, nthreads=cores, a=pp["a"], b=pp["b"], dc=pp["dc"],
              f0=pp["f0"], vplv=pp["vpl"], taudot=pp["taudot"], sigdot=pp["sigdot"])
    for _ in range(args.warmup):
        R.rkck(y0, 0.0, 1e5)
    t = time.perf_counter()
    for _ in range(args.steps):
        R.rkck(y0, 0.0, 1e5)
    t = time.perf_counter() - t
    bytes_attempt = 6.0 * ((Hs.body.size + Hn.body.size) * 8 + 2 * 2 * n * 8)
    v = args.steps * bytes_attempt / t / 1e9
    out_line({
        "impl": "reference", "metric": "H-matvec GB/s", "value": round(v, 3), "unit": "GB/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(t / args.steps * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded 3D planar thrust, Okada half space)",
        "config": {"workload": f"{w.name}: 3dph Okada half space, {n} elements, 2 H-matrices (s,n), "
                               f"ACA eps {w.eps_h}, one Cash-Karp attempt per step (12 products)",
                   "elements": n, "storage": "f64", "products_per_step": 12},
        "cpu_baseline": {"value": round(v, 3), "unit": "GB/s", "cores": cores, "kind": "port",
                         "sample": f"{args.steps} Cash-Karp attempts on the oracle's own ACA+ H-matrices "
                                   f"(setup {t_setup:.1f} s), OpenMP products on all host cores"},
        "e2e": {"value": round(v, 3), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    })


def run_kernels_mode(args):
    """One small run of every kernel outside the product's phases, sized for
    an ncu capture: assembly of both H-matrices of the Okada plane at
    imax x jmax (aca_plus, dense_fill), four Cash-Karp attempts (rk_prepare,
    p3_rk), 60 steps of the device time loop (cycle_*) and a short proposer
    fit on their trace (mlp_*).  Prints one JSON line of wall times; it is no
    bench line."""
    import hbi_gb300 as H
    from hbi_gb300 import configs, proposer
    w = configs.c2_3dph(args.imax, args.jmax)
    ctl_s, ctl_n = H.Ctl(w.nd), H.Ctl(w.nd)
    t0 = time.perf_counter()
    lf_s = H.LeafMtxp(ctl_s, w.geometry("s"), w.eps_h)
    lf_n = H.LeafMtxp(ctl_n, w.geometry("n"), w.eps_h)
    lh_s, lh_n = H.LHp(lf_s, ctl_s, args.store), H.LHp(lf_n, ctl_n, args.store)
    t1 = time.perf_counter()
    ndc, lodc = H.HACApK_gen_lattice_vector(ctl_s)
    y0, p = w.initial_state(lodc)
    rk = H.RK(lh_s, lh_n, evlaw=w.evlaw, scale=w.scale, a=p["a"], b=p["b"], dc=p["dc"], f0=p["f0"], vpl=p["vpl"])
    rk.set_state(y0)
    for _ in range(4):
        rk.attempt_async(1e5, 1e-5)
    rk.check_error()
    c = H.Cycle(rk, p["vel"], w.ds_area[lodc - 1], eps_r=1e-6)
    t2 = time.perf_counter()
    st = c.run(k_limit=60)
    t3 = time.perf_counter()
    X, T = proposer.training_set(c.trace())
    wts, hist = proposer.train(X, T, epochs=3, min_steps=20)
    t4 = time.perf_counter()
    c.close(); rk.close()
    for o in (lh_s, lh_n, lf_s, lf_n, ctl_s, ctl_n):
        o.close()
    print(json.dumps({"mode": "kernels", "workload": f"{w.name}: {w.nd} elements, {args.store} stores",
                      "assembly_s": round(t1 - t0, 3), "loop_steps": st["k"], "loop_s": round(t3 - t2, 3),
                      "proposer_samples": int(len(T)), "proposer_fit_s": round(t4 - t3, 3),
                      "proposer_loss": float(hist[-1])}))


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.mode == "matvec":
        run_matvec_mode(args)
    elif args.mode == "ensemble":
        run_ensemble_mode(args)
    elif args.mode == "kernels":
        run_kernels_mode(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
