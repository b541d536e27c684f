"""The tensor-core (tcgen05) path of the ensemble product: one BF16 MMA with
FP32 accumulation in tensor memory against the CPU product of the same BF16
values (exact products, FP32 sums: 1e-5 relative)."""
import numpy as np
import pytest

import hbi_gb300 as H

pytestmark = pytest.mark.gpu


def bf16_bits(x):
    """Round-to-nearest-even float32 -> bfloat16 bit patterns, and their values."""
    u = np.asarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)
    return r, (r.astype(np.uint32) << 16).view(np.float32)


def test_umma_bf16_matches_cpu():
    rng = np.random.default_rng(0)
    a_bits, a = bf16_bits(rng.standard_normal((128, 16)))
    b_bits, b = bf16_bits(rng.standard_normal((64, 16)))
    d = H.umma_probe(a_bits, b_bits, 0)
    ref = a.astype(np.float64) @ b.astype(np.float64).T
    assert np.allclose(d, ref, rtol=1e-5, atol=1e-5 * np.abs(ref).max())
