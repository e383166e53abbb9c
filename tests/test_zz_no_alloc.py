"""The allocation-free synthesis entry point, through the C ABI.

aeolus_synthesize_noalloc is for callers that cannot allocate device memory
(FFI hosts without a device allocator, code that must avoid the implicit
synchronisation of cudaMalloc/cudaFree): it runs the FP64 Gauss synthesis on
a fixed scratch array inside the library.  It must give the same grid values
as aeolus_synthesize with a caller-provided workspace, call after call, and
reject batches whose scratch would exceed the fixed size.  This file is
collected last so that a failure here comes after every other test.
"""
import ctypes

import numpy as np
import pytest
import torch

from aeolus_gb300 import _lib, workloads as W
from aeolus_gb300.ops import Plan, synthesize
from helpers import rel_l2

pytestmark = pytest.mark.gpu


def _noalloc(plan, coeffs):
    c = coeffs.contiguous()
    out = torch.empty((c.shape[0], plan.n_points), dtype=torch.float64, device=c.device)
    stream = ctypes.c_void_p(torch.cuda.current_stream(c.device).cuda_stream)
    status = _lib.load().aeolus_synthesize_noalloc(plan.handle, ctypes.c_void_p(c.data_ptr()),
                                                   ctypes.c_void_p(out.data_ptr()), c.shape[0], stream)
    return status, out


def test_noalloc_matches_workspace_synthesis_twice():
    plan = Plan.gauss(192, 384, 127)
    rng = np.random.default_rng(42)
    for call in range(2):  # the second call reuses the scratch the first one left
        a = np.stack([W.random_spectrum(rng, 127, -1.5, 1.0, zero_monopole=False) for _ in range(4 + call)])
        coeffs = torch.as_tensor(a, device="cuda")
        status, out = _noalloc(plan, coeffs)
        assert status == _lib.OK, _lib.load().aeolus_last_error()
        ref = synthesize(plan.id, coeffs)
        torch.cuda.synchronize()
        for b in range(a.shape[0]):
            assert rel_l2(out[b].cpu().numpy(), ref[b].cpu().numpy()) < 1e-12


def test_noalloc_rejects_oversized_batch_and_split_plans():
    plan = Plan.gauss(192, 384, 127)
    big = torch.zeros((64, 128, 128), dtype=torch.complex128, device="cuda")
    status, _ = _noalloc(plan, big)
    assert status == _lib.ERR_WORKSPACE
    assert b"16 MiB" in _lib.load().aeolus_last_error()
    split = Plan.gauss(32, 64, 21)
    split.set_precision(_lib.PREC_SPLIT_BF16)
    status, _ = _noalloc(split, torch.zeros((1, 22, 22), dtype=torch.complex128, device="cuda"))
    assert status == _lib.ERR_ARG
