"""The tensor-core kernels' bounded waits: a wait that runs out ends the call with QXG_ERR_TIMEOUT
and leaves the GPU usable.

The test hook qxg_options.tc_stall_test makes the first CTA of every tensor-core GEMM (and of
every tensor-core join) issue no operand copies, so its MMA issuer (the join's splitters) waits on
a barrier that nothing completes; with a short poll
limit (qxg_options.tc_wait_limit) the wait gives up, the CTA's other warps give up or see the
abort, and the kernel frees its tensor memory and returns.  No copy is left in flight (the
stalled producer issued none; the waits for copies in flight keep the full limit), no fault or
trap is raised.  The host reads the programme's timeout word after the call.  A second call on
the same handle must time out again (the word was cleared, not left stale), and a fresh programme
on the same GPU must then return correct results.
"""
from collections import OrderedDict

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _tc_programme(q, nm=9, nk=6, nn=5, seed=3):
    rng = np.random.default_rng(seed)
    la = list(range(1, nm + 1)) + list(range(30, 30 + nk))
    lb = list(range(30, 30 + nk)) + list(range(60, 60 + nn))
    lc = list(range(1, nm + 1)) + list(range(60, 60 + nn))
    A = rng.standard_normal((2,) * len(la)) + 1j * rng.standard_normal((2,) * len(la))
    B = rng.standard_normal((2,) * len(lb)) + 1j * rng.standard_normal((2,) * len(lb))
    cmds = [q.Load("a", "data_1", A.shape), q.Load("b", "data_2", B.shape),
            q.Ncon("c", tuple(lc), "a", tuple(la), "b", tuple(lb)), q.Save("output", "c")]
    prog = q.Programme.from_commands(cmds, OrderedDict([("data_1", A), ("data_2", B)]), 0)
    letters = {l: chr(97 + i) for i, l in enumerate(sorted(set(la) | set(lb)))}
    sub = lambda ls: "".join(letters[l] for l in ls)
    ref = np.einsum(f"{sub(la)},{sub(lb)}->{sub(lc)}", A, B).reshape(-1, order="F")
    return prog, ref


# candidate 1: the first fused X gather; 99: the last candidate, the X-planes variant
@pytest.mark.parametrize("candidate", [1, 99])
def test_expired_wait_reports_timeout_and_gpu_stays_usable(q, gpu_lib, candidate):
    prog, ref = _tc_programme(q)
    with q.Executor(prog, precision="split_tf32", tc_tuning=candidate, tc_wait_limit=1 << 14,
                    tc_stall_test=True) as ex:
        for _ in range(2):
            with pytest.raises(q.QXGError) as e:
                ex.amplitudes([""])
            assert e.value.code == -5, str(e.value)
            assert "gave up" in str(e.value)
    with q.Executor(prog, precision="split_tf32", tc_tuning=candidate) as ex:
        got = ex.amplitudes([""])[0]
        assert ex.info()["num_steps_tensor_core"] == 1
    assert np.max(np.abs(got - ref)) / np.max(np.abs(ref)) <= 5e-6


def test_short_wait_limit_alone_does_not_fail_good_calls(q, gpu_lib):
    """The poll limit only bounds waits: a programme with a smaller limit than the default but no
    stall still returns the right result (its waits complete long before the limit)."""
    prog, ref = _tc_programme(q, seed=4)
    with q.Executor(prog, precision="split_tf32", tc_tuning=1, tc_wait_limit=1 << 18) as ex:
        got = ex.amplitudes([""])[0]
    assert np.max(np.abs(got - ref)) / np.max(np.abs(ref)) <= 5e-6


def test_expired_join_wait_reports_timeout_and_gpu_stays_usable(q, gpu_lib):
    """The tensor-core join's waits: with the stall hook its first CTA's loader issues nothing, the
    splitters' waits give up, the MMA issuer and the drain warps give up in turn; the call returns
    QXG_ERR_TIMEOUT twice, and a fresh programme returns the right result."""
    from test_gpu_split import join_programme
    prog, ref = join_programme(q, 12, 5, 5, 3, seed=77)
    with q.Executor(prog, precision="split_tf32", tc_wait_limit=1 << 14, tc_stall_test=True) as ex:
        for _ in range(2):
            with pytest.raises(q.QXGError) as e:
                ex.amplitudes([""])
            assert e.value.code == -5, str(e.value)
        assert "tensor-core join" in ex.explain(2)
    with q.Executor(prog, precision="split_tf32") as ex:
        got = ex.amplitudes([""])[0]
    assert np.max(np.abs(got - ref)) / np.max(np.abs(ref)) <= 5e-6
