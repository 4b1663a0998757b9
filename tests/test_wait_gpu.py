"""Bounded waits give up with an error status instead of hanging (GPU test).

The pipelined step kernels wait on mbarriers with a time limit; a wait that runs out raises the
device error flag that adfwi_acoustic_status reports and the block exits. The self-test entry
point waits, through the same wait loop, on a barrier phase that nothing completes: the flag must
read 1 after the limit, the call must return in about that time, and the context must still run
a solve afterwards.
"""
import time

import pytest
import torch

import adfwi_gb300 as A
from adfwi_gb300 import _native as N
from _cases import acoustic_problem

pytestmark = pytest.mark.gpu


def test_wait_that_nothing_completes_times_out_with_status():
    flag = torch.zeros(1, dtype=torch.int32, device="cuda:0")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    N.wait_selftest(20_000_000, flag)  # 20 ms
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    assert int(flag.item()) == 1
    assert 0.015 <= dt < 1.0, dt
    # the context is still usable: a solve runs and reports a clean status
    model, survey, prop = acoustic_problem(A, ns=2, nt=60, seed=3)
    rec = prop.forward()
    assert torch.isfinite(rec["p"]).all()


def test_wait_selftest_rejects_bad_arguments():
    flag = torch.zeros(1, dtype=torch.int32, device="cuda:0")
    with pytest.raises(RuntimeError):
        N.wait_selftest(0, flag)
    with pytest.raises(RuntimeError):
        N.wait_selftest(3_000_000_000, flag)
