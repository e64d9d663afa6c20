"""t9gb_ufield_noalloc: the allocation-free mutual-field entry point.

Callers that may not allocate device memory when they need the field (hosts
that own every allocation, code inside a CUDA-graph stream capture, real-time
loops that forbid allocator calls) use this entry point; its only working
memory is a static device array inside the library.  The test calls it
through the C ABI twice in a row, with different dipoles, and checks each
result against the existing entry point t9gb_ufield on a context configured
for the same damped (non-Ewald) field and against the FP64 oracle's
non-Ewald ufield (every mutual scale of the water box is 1), within the
field tolerance used by the other GPU tests.  This file is collected last so
a failure here leaves every other test already run.
"""
import ctypes as C

import numpy as np
import pytest

from gpu_util import cpu, engine_for, rel_err

pytestmark = pytest.mark.gpu
FIELD_RTOL = 5.0e-5


def test_noalloc_ufield_matches_context_entry(gpu_lib, tg, oracle):
    import torch

    abi = gpu_lib
    lib = abi.load()
    s = tg.systems.make_config("water648")
    cutoff = 7.0
    e = engine_for(s, use_ewald=0, aewald=0.0, ewald_cutoff=cutoff, nfft=(0, 0, 0))
    box = (C.c_double * 3)(*[float(v) for v in s.box])
    dev = "cuda"
    xyz = torch.tensor(s.xyz, dtype=torch.float32, device=dev).contiguous()
    pdamp = torch.tensor(s.pdamp, dtype=torch.float32, device=dev).contiguous()
    thole = torch.tensor(s.thole, dtype=torch.float32, device=dev).contiguous()
    assert np.all(s.excl_scale[:, 3] == 1.0)
    o = oracle.OracleSystem(s, use_ewald=0, cutoff=cutoff)
    rng = np.random.default_rng(3)
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        ud = rng.normal(scale=0.05, size=(s.n, 3))
        up = rng.normal(scale=0.05, size=(s.n, 3))
        ref, refp = e.ufield(ud, up)
        tud = torch.tensor(ud, dtype=torch.float32, device=dev).contiguous()
        tup = torch.tensor(up, dtype=torch.float32, device=dev).contiguous()
        f = torch.full((s.n, 3), float("nan"), device=dev)
        fp = torch.full((s.n, 3), float("nan"), device=dev)
        rc = lib.t9gb_ufield_noalloc(
            s.n, box, cutoff, C.c_void_p(xyz.data_ptr()), C.c_void_p(pdamp.data_ptr()),
            C.c_void_p(thole.data_ptr()), C.c_void_p(tud.data_ptr()), C.c_void_p(tup.data_ptr()),
            C.c_void_p(f.data_ptr()), C.c_void_p(fp.data_ptr()), C.c_void_p(stream),
        )
        assert rc == abi.T9GB_OK, lib.t9gb_status_string(rc)
        torch.cuda.synchronize()
        assert rel_err(cpu(f), cpu(ref)) < FIELD_RTOL, f"call {call}"
        assert rel_err(cpu(fp), cpu(refp)) < FIELD_RTOL, f"call {call}"
        of, ofp = o.ufield(ud, up)
        print(f"call {call}: vs oracle {rel_err(cpu(f), of):.2e} / {rel_err(cpu(fp), ofp):.2e}")
        assert rel_err(cpu(f), of) < FIELD_RTOL, f"call {call}"
        assert rel_err(cpu(fp), ofp) < FIELD_RTOL, f"call {call}"


def test_noalloc_rejects_oversize(gpu_lib):
    abi = gpu_lib
    lib = abi.load()
    n = abi.T9GB_NOALLOC_MAX_ATOMS + 1
    dummy = C.c_void_p(1)
    rc = lib.t9gb_ufield_noalloc(n, None, 7.0, dummy, dummy, dummy, dummy, dummy, dummy, dummy, None)
    assert rc == abi.T9GB_TOO_LARGE
    assert b"fixed-capacity" in lib.t9gb_status_string(rc)
