"""Bounded device waits of the one-launch-per-slab pipelined Chebyshev kernel.

In that mode a tile waits (acquire loads, bounded polls) until every row
group whose rows it reads has published the previous step.  The test makes
such a wait run out without any fault: LARGETB_TEST_STALL_TILE names a tile
whose flags are never published (a flag that nothing sets) and
LARGETB_TEST_WAIT_LIMIT shortens the poll limit to a few milliseconds.  The
kernel must then stop early and return, tb_density must report
TB_ERR_TIMEOUT with a message naming the wait, and the same context must give
the undisturbed result on the next call.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_neighbour_wait_times_out_and_context_recovers(gpu, monkeypatch):
    T = gpu
    m = T.model_cristobalite(2, 2, 2, sigma_ang=0.05, seed=1001)
    with T.Context(M=60, precision=T.PREC_FP32, fp32_kernel=T.FP32_PIPELINED, column_block=256,
                   device=0) as c:
        c.set_model(m)
        ref = c.density()
        assert ref["report"]["step_kernel"] == T.FP32_PIPELINED
        monkeypatch.setenv("LARGETB_TEST_WAIT_LIMIT", "4096")
        monkeypatch.setenv("LARGETB_TEST_STALL_TILE", "0")
        with pytest.raises(T.TbError) as e:
            c.density()
        assert e.value.status == T.api.TB_ERR_TIMEOUT
        assert "neighbour-flag wait ran out" in str(e.value)
        monkeypatch.delenv("LARGETB_TEST_WAIT_LIMIT")
        monkeypatch.delenv("LARGETB_TEST_STALL_TILE")
        again = c.density()
    # the recurrence is deterministic: the recovered context gives the same bits
    np.testing.assert_array_equal(again["q"], ref["q"])
    assert again["e_band"] == ref["e_band"]
