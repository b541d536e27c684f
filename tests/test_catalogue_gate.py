"""The accuracy gate on event catalogues (hbi_gb300.catalogue), host only.

Synthetic catalogues with the structure of the 200,000-triangle rough fault's
first earthquake: a train of slip-rate flickers (mean slip ~1e-7 m) before
the main rupture (mean slip 1.4 m).  Merged or missing flickers with onsets
that still match do not fail the gate; a missing or shifted earthquake, a
wrong earthquake slip or a flicker with no counterpart does.
"""
import copy

import numpy as np

from hbi_gb300.catalogue import GATE, catalogue_gate

T0 = 6.1301243746e8  # s: the first flicker of the FP64 run


def _cat():
    ev = [dict(id=i + 1, onset=T0 + 7.0 * i, moment=1e-7 * (1 + 0.3 * i)) for i in range(14)]
    ev.append(dict(id=15, onset=T0 + 170.0, moment=1.4115))
    return {"events": ev, "slip": np.linspace(0.1, 2.0, 50)}


def test_identical_catalogues_pass():
    g = catalogue_gate(_cat(), _cat())
    assert g["pass"] and g["failures"] == [] and g["earthquakes"] == [1, 1]


def test_merged_and_missing_flickers_pass():
    m = _cat()
    del m["events"][9]     # two flickers merged into one
    del m["events"][0]     # a flicker just above velth not sampled
    for e in m["events"]:
        e["onset"] += 2.4  # onsets shifted by seconds (4e-9 relative)
    m["events"][-1]["moment"] *= 1 + 2e-6
    g = catalogue_gate(_cat(), m)
    assert g["pass"], g["failures"]
    assert g["events_all"] == [15, 13] and g["earthquakes"] == [1, 1]


def test_missing_earthquake_fails():
    m = _cat()
    m["events"].pop()
    g = catalogue_gate(_cat(), m)
    assert not g["pass"] and any("earthquakes" in f for f in g["failures"])


def test_earthquake_slip_and_onset_are_bounded():
    m = _cat()
    m["events"][-1]["moment"] *= 1 + 2 * GATE
    assert not catalogue_gate(_cat(), m)["pass"]
    m = _cat()
    m["events"][-1]["onset"] *= 1 + 2 * GATE
    g = catalogue_gate(_cat(), m)
    assert not g["pass"] and any("onset" in f for f in g["failures"])


def test_unmatched_flicker_and_slip_field_fail():
    m = _cat()
    m["events"].insert(0, dict(id=0, onset=T0 * 0.5, moment=1e-7))
    assert not catalogue_gate(_cat(), m)["pass"]
    m = copy.deepcopy(_cat())
    m["slip"] = m["slip"] * (1 + 2 * GATE)
    g = catalogue_gate(_cat(), m)
    assert not g["pass"] and any("slip field" in f for f in g["failures"])
