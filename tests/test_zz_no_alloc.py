"""The no-allocation adjoint entry point (collected last on purpose).

``tsg_epg_adjoint_noalloc`` serves callers that cannot allocate device
memory (a reconstruction service with its memory planned at start-up, a
framework whose caching allocator owns the GPU): its scratch lives in one
static device array. This checks it against the allocating entry point,
``tsg_epg_adjoint``, through the C ABI, on two calls in a row (the second
sees the array as the first left it), and that an oversized problem is
rejected. It is written to pass alone in a fresh process as well as after
the rest of the suite.
"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest
import torch

from tests.helpers import draw_tissue, max_rel

pytestmark = pytest.mark.gpu

GRAD_TOL = 1e-4
NAMES = ("t1_ms", "t2_ms", "m0", "b1", "inversion", "flip_rad", "duration_s")


def _case(device, voxels=300, pulses=120, states=10, seed=17):
    from torchsim_gb300 import engine
    from torchsim_gb300.sequence import mrf_events, program_for

    rng = np.random.default_rng(seed)
    ev = mrf_events(rng.uniform(5, 70, pulses).astype(np.float32),
                    rng.uniform(8, 15, pulses).astype(np.float32), TI_ms=10.0)
    t1, t2, b1 = draw_tissue(seed, voxels)
    m0 = rng.uniform(0.5, 1.5, voxels).astype(np.float32)
    inv = rng.uniform(0.85, 1.0, voxels).astype(np.float32)
    prog = program_for(ev, device)
    tissue = engine.tissue_maps(device, voxels, t1, t2, m0, b1, inv)
    cot = torch.from_numpy(rng.standard_normal((voxels, ev.outputs)).astype(np.complex64))
    return prog, tissue, cot.to(device), ev


def _zeros(device, voxels, events):
    g = {n: torch.zeros(voxels, device=device) for n in NAMES[:5]}
    g["flip_rad"] = torch.zeros((1, events), device=device)
    g["duration_s"] = torch.zeros((1, events), device=device)
    return g


def _noalloc(lib, prog, tissue, states, seed, grads):
    from torchsim_gb300 import _native, engine

    g = _native.Gradients(*[grads[n].data_ptr() for n in NAMES])
    t = tissue.struct()
    return lib.tsg_epg_adjoint_noalloc(prog.handle, ctypes.byref(t), tissue.voxels, states,
                                       seed.data_ptr(), _native.LAYOUT_COMPLEX_IJ, ctypes.byref(g),
                                       None, engine._stream())


def test_noalloc_adjoint_matches_allocating_entry(built_library, cuda):
    from torchsim_gb300 import _native, engine

    states = 10
    prog, tissue, seed, ev = _case(cuda, states=states)
    # The existing entry point, with buffers the caller allocates.
    c, ck, _ = engine.adjoint_plan(prog, tissue.voxels, states)
    ckpt = torch.empty(ck // 4, dtype=torch.float32, device=cuda)
    engine.forward_checkpointed(prog, tissue, states, c, ckpt)
    expected = engine.adjoint(prog, tissue, states, seed, ckpt, c,
                              _zeros(cuda, tissue.voxels, ev.events))
    for call in range(2):
        got = _zeros(cuda, tissue.voxels, ev.events)
        _native.check(_noalloc(built_library, prog, tissue, states, seed, got))
        torch.cuda.synchronize()
        for name in NAMES:
            ref = expected[name].cpu().numpy()
            assert max_rel(got[name].cpu().numpy(), ref) <= GRAD_TOL, (call, name)


def test_noalloc_rejects_beyond_its_array(built_library, cuda):
    from torchsim_gb300 import _native

    cap = built_library.tsg_static_scratch_bytes()
    assert cap == 32 * 1024 * 1024
    prog, tissue, seed, ev = _case(cuda, voxels=40000, pulses=120, states=10)
    got = _zeros(cuda, tissue.voxels, ev.events)
    rc = _noalloc(built_library, prog, tissue, 10, seed, got)
    assert rc == _native.TSG_ERR_CAPACITY
    assert b"static array holds" in built_library.tsg_last_error()
    assert not any(bool(v.any()) for v in got.values())
