"""The allocation-free sum (pd_reduce_sum_static) against the context-based
one (pd_reduce_sum), through the C ABI.

pd_reduce_sum_static is for callers that cannot allocate device memory: it
takes no context and keeps its partial sums in a fixed array inside the
library.  This file is collected last so that a run stopping at the first
failure has already run every other test; it passes alone in a fresh process
and after the rest of the suite.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# both sums are deterministic but group the terms differently
RTOL = 1e-12


def test_static_sum_matches_context_sum_twice():
    import torch

    from pd_gpu1_gb300 import engine as E
    from pd_gpu1_gb300._lib import lib

    L = lib()
    p = E.derive_params(2, 1, 2, 1e-7, 1, 5e-4, 0.0, 5e-4, 0.02, 0.015, 0.0, 192e9, 1 / 3, 8000.0, 0.04472)
    rng = np.random.default_rng(5)
    stream = torch.cuda.current_stream().cuda_stream
    with E.Engine(p) as eng:
        n = p.N
        out = torch.full((2,), float("nan"), dtype=torch.float64, device="cuda")
        for call in range(2):
            vals = rng.standard_normal(n) * 10.0 ** rng.uniform(-3, 3, n)
            eng.set("UX", vals)
            ref = eng.sum("UX")
            ptr, count = eng.device_ptr("UX")
            rc = L.pd_reduce_sum_static(ptr, count, out.data_ptr() + 8 * call, stream)
            assert rc == 0
            torch.cuda.synchronize()
            got = float(out[call].item())
            assert got == pytest.approx(ref, rel=RTOL, abs=RTOL * np.abs(vals).sum())
            assert got == pytest.approx(float(np.sum(vals)), rel=1e-10, abs=1e-10 * np.abs(vals).sum())
        # a larger input from torch memory, and the size limit
        big = torch.randn(5_000_003, dtype=torch.float64, device="cuda")
        rc = L.pd_reduce_sum_static(big.data_ptr(), big.numel(), out.data_ptr(), stream)
        assert rc == 0
        torch.cuda.synchronize()
        assert float(out[0].item()) == pytest.approx(float(big.sum().item()), rel=1e-9, abs=1e-9 * 5e6)
        assert L.pd_reduce_sum_static(big.data_ptr(), 33_554_432 + 1, out.data_ptr(), stream) == -1
