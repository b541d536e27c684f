"""Comparison of two event catalogues of the time loop (main_LH.f90:
1338-1388) and of their slip fields, for the accuracy gate of the mixed form
against the plain FP64 form: slip and event timing within 1e-3 relative.

The reference's event rule starts an event when the maximum slip rate
exceeds velth (1 cm/s) and ends it when it falls below velth/2; the event
slip is the mean slip accumulated in between.  Besides the earthquakes it
also lists the brief slip-rate flickers of a nucleating rupture (mean slip
~1e-7 m).  Whether one of them peaks just above velth, or whether the dip
between two of them just reaches velth/2 at a step end, depends on where the
accepted steps end, so their count is ill-conditioned: on the 200,000-
triangle rough fault the FP64 run lists 14 flickers before its first
earthquake and the FP32 run 13: between two flickers the maximum slip rate
sampled at the step ends bottoms out at 4.51 mm/s in the FP64 run (below
velth/2, so the first flicker ends and another starts) and at 5.08 mm/s in
the FP32 run (the two are one event).  The gate therefore pairs the
earthquakes -- events with at least MAIN_FRAC of the largest event's slip --
one to one (same count, onset and slip within GATE), requires every event,
flickers included, to have an onset within GATE of one in the other
catalogue, and bounds the slip fields' difference; every difference is
listed.
"""
import numpy as np

GATE = 1e-3       # relative error bound of slip and event timing
MAIN_FRAC = 1e-2  # an earthquake: an event with at least this fraction of the largest event's slip


def catalogue_gate(plain, mixed):
    """plain, mixed: {"events": [{"id", "onset", "moment", ...}], "slip": array}
    (Cycle.events() and the slip of Cycle.fields()).  Returns the gate's
    verdict ("pass"), the listed failures and the largest errors."""
    ep, em = plain["events"], mixed["events"]
    big = max((abs(e["moment"]) for e in ep), default=0.0)
    main_p = [e for e in ep if abs(e["moment"]) >= MAIN_FRAC * big]
    main_m = [e for e in em if abs(e["moment"]) >= MAIN_FRAC * big]
    fails = []
    if len(main_p) != len(main_m):
        fails.append(f"earthquakes (slip >= {MAIN_FRAC:g} of the largest): plain {len(main_p)}, mixed {len(main_m)}")
    on_err, sl_err, on_abs = 0.0, 0.0, 0.0
    for a, b in zip(main_p, main_m):
        eo = abs(b["onset"] - a["onset"]) / a["onset"]
        es = abs(b["moment"] - a["moment"]) / abs(a["moment"])
        on_err, sl_err, on_abs = max(on_err, eo), max(sl_err, es), max(on_abs, abs(b["onset"] - a["onset"]))
        if eo > GATE:
            fails.append(f"earthquake {a['id']}: onset {a['onset']:.9e} s vs {b['onset']:.9e} s (rel {eo:.2e})")
        if es > GATE:
            fails.append(f"earthquake {a['id']}: slip {a['moment']:.6e} m vs {b['moment']:.6e} m (rel {es:.2e})")

    def nearest(e, other):
        return min((abs(o["onset"] - e["onset"]) / e["onset"] for o in other), default=float("inf"))

    all_err = max([nearest(e, em) for e in ep] + [nearest(e, ep) for e in em], default=0.0)
    if all_err > GATE:
        fails.append(f"an event without a counterpart within {GATE:g} in the other catalogue (rel {all_err:.2e})")
    slip_err = float(np.linalg.norm(mixed["slip"] - plain["slip"]) / np.linalg.norm(plain["slip"]))
    if not slip_err <= GATE:
        fails.append(f"slip field at the window's end: rel {slip_err:.2e}")
    return {"pass": not fails, "bound": GATE, "failures": fails,
            "earthquakes": [len(main_p), len(main_m)], "events_all": [len(ep), len(em)],
            "earthquake_onset_rel_err_max": on_err, "earthquake_onset_abs_s_max": round(on_abs, 3),
            "earthquake_slip_rel_err_max": sl_err, "every_onset_rel_err_max": all_err,
            "slip_rel_err_at_window_end": slip_err}
