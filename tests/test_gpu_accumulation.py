"""The tensor cores' FP32 accumulation against the error bound of the BF16 candidate test.

The BF16 mode keeps a pair as a candidate when its Gram-form squared distance is within
(eps' + a_i + a_j)^2 + q_i + q_j, where q bounds each row's share of the accumulation
error of the tensor-core dot product (gram_bf16.cu, bf16_gamma: at most 2^-19 relative
error per addition of the FP32 accumulator, plus the rounding of the norms and of the
final combination).  That model of undocumented hardware is what keeps the edge set
exact, so it is measured here: one tile pair goes through the production Gram kernel
(rnng_gram_probe_bf16), and its raw accumulators are compared with the exact dot products
of the BF16 operands it was given.  The rows are built to stress the accumulator: mixed
signs, exponents spread over 2^-10 .. 2^10 inside each row, column rows equal to row-tile
rows with half the signs flipped (heavy cancellation), at several magnitudes."""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

WORST = {}


def stressed_rows(d, scale_exp, seed):
    rng = np.random.default_rng(seed)
    x = rng.uniform(1.0, 2.0, (256, d)) * rng.choice([-1.0, 1.0], (256, d)) * 2.0 ** rng.integers(-10, 11, (256, d))
    flip = np.where(rng.random((128, d)) < 0.5, -1.0, 1.0)
    x[128:] = x[:128] * flip * (1.0 + 2.0 ** -7 * rng.standard_normal((128, d)))
    x[200:] = rng.uniform(-1.0, 1.0, (56, d)) * 2.0 ** 10  # and some unrelated rows
    return (x * 2.0 ** scale_exp).astype(np.float32)


@pytest.mark.parametrize("d", [64, 128, 192, 256])
@pytest.mark.parametrize("scale_exp", [-50, -20, 0, 20, 45])
def test_tensor_core_accumulation_within_bound(ctx, d, scale_exp):
    x = stressed_rows(d, scale_exp, seed=1000 * d + scale_exp + 60)
    G, Xb, info = ctx.gram_probe_bf16(x)
    A = Xb[:128].astype(np.float64)
    B = Xb[128:].astype(np.float64)
    # products of BF16 values are exact in float64; fsum rounds their sum once
    exact = np.array([[math.fsum(A[i] * B[j]) for j in range(128)] for i in range(128)])
    err = 2.0 * np.abs(G.astype(np.float64) - exact)
    bound = info[:128, 2].astype(np.float64)[:, None] + info[128:, 2].astype(np.float64)[None, :]
    assert np.all(bound > 0)
    ratio = float(np.max(err / bound))
    WORST[(d, scale_exp)] = ratio
    print(f"d={d} scale=2^{scale_exp}: max |2 (g - exact)| / (q_i + q_j) = {ratio:.3e}")
    assert ratio < 1.0
    # the norms the test uses are the BF16 rows' own (to FP32 rounding)
    norms = (Xb.astype(np.float64) ** 2).sum(1)
    assert np.allclose(info[:, 0], norms, rtol=1e-5)
