"""The allocation-free product, hbi_adot_lattice_hyp_noalloc, against the
allocating one, hbi_adot_lattice_hyp_dev, through the C ABI.

The no-alloc entry point serves callers that cannot allocate device memory
when they multiply (device memory owned by another allocator or a fixed
budget, or a time loop that must stay clear of cudaMalloc and its device-wide
synchronisation).  Its scratch is a 16 MiB array inside the library, shared by
all calls, so two calls in a row must each give the same product as the
allocating path, bit for bit (same kernels, schedules and summation order) --
the second call must not see stale data from the first.

This file is collected last so that a failure here leaves every other test
already run; it also passes on its own in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

import hbi_gb300 as H
from gpu_cases import case, product_geometry

pytestmark = pytest.mark.gpu


def _noalloc(lh, d_au, d_u, stream):
    return H.lib().hbi_adot_lattice_hyp_noalloc(C.c_void_p(d_au), lh.h, C.c_void_p(d_u), C.c_void_p(stream))


@pytest.mark.parametrize("kind,store,tol", [("3dph", "f64", 1e-12), ("3dph", "f32", 1e-5), ("3dnt", "bf16", 2e-2)])
def test_noalloc_matches_allocating_product(kind, store, tol):
    import torch
    prob, n, g, w, eps = case(kind)
    ctl = H.Ctl(n)
    lf = H.LeafMtxp(ctl, product_geometry(prob, n, g, w, "s"), eps)
    lh = H.LHp(lf, ctl, store)
    l64 = H.LHp(lf, ctl, "f64")
    st = torch.cuda.Stream()
    gen = torch.Generator(device="cuda").manual_seed(5)
    for call in range(2):  # two calls in a row share the scratch array
        u = torch.randn(n, dtype=torch.float64, device="cuda", generator=gen)
        ref = torch.empty(n, dtype=torch.float64, device="cuda")
        out = torch.full((n,), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        lh.matvec_dev(ref.data_ptr(), u.data_ptr(), st.cuda_stream)
        rc = _noalloc(lh, out.data_ptr(), u.data_ptr(), st.cuda_stream)
        assert rc == 0, H.lib().hbi_last_error()
        st.synchronize()
        assert H.lib().hbi_lh_check_error(lh.h) == 0
        r, o = ref.cpu().numpy(), out.cpu().numpy()
        assert np.all(np.isfinite(o))
        # the same kernels, warp schedules and summation order as the
        # allocating path: any stale scratch would show as a difference
        assert np.array_equal(o, r), (call, np.linalg.norm(o - r) / np.linalg.norm(r))
        # and the product itself is the one of the factors (storage tolerance)
        r64 = l64.matvec(u.cpu().numpy())
        assert np.linalg.norm(o - r64) <= tol * np.linalg.norm(r64)


def test_noalloc_rejects_operators_beyond_its_scratch():
    import torch
    n = 600_000  # 2D antiplane: the row-group partials alone exceed 16 MiB in FP64
    prob, _, g, w, eps = case("2dvs", n)
    ctl = H.Ctl(n)
    lf = H.LeafMtxp(ctl, product_geometry(prob, n, g, w, "s"), 1e-4)
    lh = H.LHp(lf, ctl, "f64")
    u = torch.ones(n, dtype=torch.float64, device="cuda")
    out = torch.zeros(n, dtype=torch.float64, device="cuda")
    rc = _noalloc(lh, out.data_ptr(), u.data_ptr(), 0)
    assert rc == -6  # HBI_ERR_LIMIT
    assert b"limit" in H.lib().hbi_last_error()
