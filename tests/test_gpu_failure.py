"""Failure handling of the kernels with bounded waits, tested without a GPU fault.

rnng_ctx_fault_drill makes the tensor-core Gram kernel's epilogue wait on a barrier that
nothing arrives on.  Its wait gives up after about one second, records the fault in the
context's fault word and raises the CTA's abort flag; the other roles stop issuing work,
drain their copies and MMAs in flight, free tensor memory and return.  The call reports
RNNG_ERR_DEVICE, and the next call on the same context works."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_gram_bounded_wait_runs_out_and_context_recovers(ctx, orc):
    import rnng_gb300
    from rnng_gb300 import synth

    x = synth.descriptor(n=5000, d=128, k=10, seed=7)
    r = synth.EPS_K2
    want = orc.eps_graph_l2(x, r)
    ctx.fault_drill(True)
    t0 = time.time()
    try:
        with pytest.raises(rnng_gb300.RnngError) as e:
            ctx.eps_graph_l2(x, r, mode="bf16")
    finally:
        ctx.fault_drill(False)
    assert e.value.code == 5 and "fault word" in str(e.value)
    assert time.time() - t0 < 30.0
    # the FP32 tiles never wait; the BF16 kernel runs again on the same context
    for mode in ("fp32", "bf16"):
        u, v, w = ctx.eps_graph_l2(x, r, mode=mode)
        assert np.array_equal(u, want[0]) and np.array_equal(v, want[1])
        assert np.array_equal(w.view(np.uint32), want[2].view(np.uint32))
