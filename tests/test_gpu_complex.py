"""GPU parity of the complex kernel (RF and receiver phases, B0, B1phase):
against the FP64 restatement of the reference's complex kernel
(src/torchsim/_epg_cpu.cpp:4216-4566) and the reference's own public outputs
recorded in the fixtures, at the stated signal tolerance."""

from __future__ import annotations

import numpy as np
import pytest
import torch

from oracle import oracle as O
from tests.helpers import max_rel, packed_complex_from_golden, packed_from_events

pytestmark = pytest.mark.gpu

SIGNAL_TOL = 1e-5
JACOBIAN_TOL = 1e-4


def _run(cuda, d, launch=None, layout_planes=False):
    from torchsim_gb300 import _native, engine
    from torchsim_gb300.sequence import PackedEvents, Program

    ev = PackedEvents(duration=np.atleast_2d(d["event_duration"]), kind=d["event_kind"],
                      flip=np.atleast_2d(d["event_flip"]), phase=np.atleast_2d(d["event_phase"]),
                      action=d["event_action"], output_index=d["event_output_index"])
    prog = Program(ev, phased=True)
    t = lambda k: torch.from_numpy(d[k]).to(cuda)
    tissue = engine.tissue_maps(cuda, d["tissue_t1_ms"].size, t("tissue_t1_ms"),
                                t("tissue_t2_ms"), t("tissue_m0"), t("tissue_b1"),
                                t("tissue_inversion_efficiency"))
    off, keep = engine.offaxis_maps(cuda, d["tissue_t1_ms"].size, t("tissue_b1_phase_rad"),
                                    t("tissue_b0_hz"))
    out = engine.forward_complex(prog, tissue, int(d["states"]), off, launch=launch)
    torch.cuda.synchronize()
    return -1j * out.cpu().numpy()


@pytest.mark.parametrize("name", ["fse_phase0", "mrf_offaxis"])
@pytest.mark.parametrize("launch", [None, (1, 10, 4), (2, 6, 4), (4, 4, 2), (5, 4, 4),
                                    (10, 2, 4), (8, 4, 4), (32, 4, 2)])
def test_complex_kernel_matches_oracle(cuda, golden, name, launch):
    d = golden(name)
    if launch is not None and launch[0] * launch[1] < int(d["states"]):
        pytest.skip("shape holds fewer orders than the case")
    got = _run(cuda, d, launch)
    ref = O.forward_complex(packed_complex_from_golden(d), "f64")
    assert max_rel(got, ref) <= SIGNAL_TOL
    assert max_rel(got, d["raw_forward"]) <= SIGNAL_TOL


def test_default_phase_fse_matches_reference_signal(cuda, golden):
    import torchsim_gb300 as ts

    d = golden("fse_phase0")
    sig = ts.fse_sim(torch.from_numpy(d["flip_deg"]), float(d["esp_ms"]),
                     torch.from_numpy(d["t1"]).to(cuda), torch.from_numpy(d["t2"]).to(cuda),
                     B1=torch.from_numpy(d["b1"]).to(cuda), states=int(d["states"]))
    assert max_rel(sig.cpu().numpy(), d["signal"]) <= SIGNAL_TOL


def test_offaxis_mrf_matches_reference_signal(cuda, golden):
    import torchsim_gb300 as ts

    d = golden("mrf_offaxis")
    tt = lambda k: torch.from_numpy(d[k]).to(cuda)
    sim = ts.MRFSimulator(flip=torch.from_numpy(d["flip_deg"]), TR=torch.from_numpy(d["tr_ms"]),
                          TI=float(d["ti_ms"]), states=int(d["states"]))
    sig = sim.simulate(T1=tt("t1"), T2=tt("t2"), B1=tt("b1"), B0=tt("b0"),
                       B1phase=tt("b1_phase"), M0=tt("m0"))
    assert max_rel(sig.cpu().numpy(), d["signal"]) <= SIGNAL_TOL
    names = tuple(str(n) for n in d["jacobian_names"])
    _, jac = sim.jacobian(names, T1=tt("t1"), T2=tt("t2"), B1=tt("b1"), B0=tt("b0"),
                          B1phase=tt("b1_phase"), M0=tt("m0"))
    for c, name in enumerate(names):
        assert max_rel(jac[:, c].cpu().numpy(), d["jacobian"][:, c]) <= JACOBIAN_TOL, name
    # The inversion-efficiency column on the complex path (a general-tangent
    # launch beside the fused sweep) against central differences of the
    # public signal.
    inv = tt("t1") * 0 + 0.9
    _, col = sim.jacobian(("T1", "inv_efficiency"), T1=tt("t1"), T2=tt("t2"), B0=tt("b0"),
                          inv_efficiency=inv)
    h = 1e-3
    up = sim.simulate(T1=tt("t1"), T2=tt("t2"), B0=tt("b0"), inv_efficiency=inv + h)
    down = sim.simulate(T1=tt("t1"), T2=tt("t2"), B0=tt("b0"), inv_efficiency=inv - h)
    fd = ((up.to(torch.complex128) - down.to(torch.complex128)) / (2 * h)).cpu().numpy()
    assert max_rel(col[:, 1].cpu().numpy(), fd) <= 1e-3


def test_default_phase_fse_jacobian_matches_reference(cuda, golden):
    import torchsim_gb300 as ts

    d = golden("fse_phase0")
    tt = lambda k: torch.from_numpy(d[k]).to(cuda)
    names = tuple(str(n) for n in d["jacobian_names"])
    _, jac = ts.fse_sim(torch.from_numpy(d["flip_deg"]), float(d["esp_ms"]), tt("t1"), tt("t2"),
                        B1=tt("b1"), states=int(d["states"]), diff=names)
    for c, name in enumerate(names):
        assert max_rel(jac[:, c].cpu().numpy(), d["jacobian"][:, c]) <= JACOBIAN_TOL, name


@pytest.mark.parametrize("launch", [None, (5, 2, 4), (4, 4, 2), (8, 4, 4)])
def test_complex_tangents_against_central_differences(cuda, golden, launch):
    """Each column against central differences of the FP64 complex oracle."""
    from torchsim_gb300 import engine
    from torchsim_gb300.sequence import PackedEvents, Program

    d = golden("mrf_offaxis")
    ev = PackedEvents(duration=np.atleast_2d(d["event_duration"]), kind=d["event_kind"],
                      flip=np.atleast_2d(d["event_flip"]), phase=np.atleast_2d(d["event_phase"]),
                      action=d["event_action"], output_index=d["event_output_index"])
    prog = Program(ev, phased=True)
    t = lambda k: torch.from_numpy(d[k]).to(cuda)
    V = d["tissue_t1_ms"].size
    tissue = engine.tissue_maps(cuda, V, t("tissue_t1_ms"), t("tissue_t2_ms"), t("tissue_m0"),
                                t("tissue_b1"), None)
    off, keep = engine.offaxis_maps(cuda, V, t("tissue_b1_phase_rad"), t("tissue_b0_hz"))
    names = ("T1", "T2", "B1", "M0")
    S = int(d["states"])
    if launch is not None and launch[0] * launch[1] < S:
        pytest.skip("shape holds fewer orders than the case")
    sig, jac = engine.forward_tangents_complex(prog, tissue, S, names, off, launch=launch)
    got = -1j * jac.cpu().numpy()
    p = packed_complex_from_golden(d)
    p.inversion = None
    keys = {"T1": "t1_ms", "T2": "t2_ms", "B1": "b1", "M0": "m0"}
    for c, name in enumerate(names):
        base = getattr(p, keys[name]).astype(np.float64)
        h = 1e-4 * np.abs(base) + 1e-6
        cols = []
        for sign in (1, -1):
            q = packed_complex_from_golden(d)
            q.inversion = None
            setattr(q, keys[name], (base + sign * h).astype(np.float32))
            cols.append(O.forward_complex(q, "f64"))
        # The perturbed inputs pass through float32: divide by the step they took.
        step = ((base + h).astype(np.float32).astype(np.float64)
                - (base - h).astype(np.float32).astype(np.float64))
        fd = (cols[0] - cols[1]) / step[:, None]
        assert max_rel(got[:, c], fd) <= 1e-3, name
    assert max_rel(-1j * sig.cpu().numpy(), O.forward_complex(p, "f64")) <= SIGNAL_TOL


def test_complex_kernel_is_deterministic_and_batch_independent(cuda):
    from torchsim_gb300 import engine
    from torchsim_gb300.sequence import fse_events, program_for

    rng = np.random.default_rng(9)
    ev = fse_events(rng.uniform(100, 180, 24).astype(np.float32), 7.0)  # refocusing at 0 deg
    assert ev.real_axis() == -1
    V, S = 3000, 48
    t1 = torch.from_numpy(rng.uniform(300, 3000, V).astype(np.float32)).to(cuda)
    t2 = torch.from_numpy(rng.uniform(10, 300, V).astype(np.float32)).to(cuda)
    b0 = torch.from_numpy(rng.uniform(-30, 30, V).astype(np.float32)).to(cuda)
    prog = program_for(ev, cuda, phased=True)
    tissue = engine.tissue_maps(cuda, V, t1, t2, None, None, None)
    off, keep = engine.offaxis_maps(cuda, V, None, b0)
    a = engine.forward_complex(prog, tissue, S, off).clone()
    b = engine.forward_complex(prog, tissue, S, off)
    assert torch.equal(a, b)
    sub = engine.tissue_maps(cuda, 17, t1[100:117], t2[100:117], None, None, None)
    off2, keep2 = engine.offaxis_maps(cuda, 17, None, b0[100:117])
    part = engine.forward_complex(prog, sub, S, off2)
    assert torch.equal(part, a[100:117])
    p = packed_from_events(ev, t1[:64].cpu().numpy(), t2[:64].cpu().numpy(), S)
    p.phase_rad = ev.phase
    p.b0_hz = b0[:64].cpu().numpy()
    ref = O.forward_complex(p, "f64")
    assert max_rel(-1j * a[:64].cpu().numpy(), ref) <= SIGNAL_TOL
