"""Generate the golden fixtures in this folder from the reference itself.

Run in a container that has the reference checkout (the argument, else
$TORCHSIM_REFERENCE, else /root/reference)
and a C++ compiler:

    python tests/golden/make_golden.py [REFERENCE_ROOT] [CASE ...]

It builds the reference's own CPU kernel with ``oracle/build_ref.sh``, imports
the reference's Python package from a temporary copy, runs its public calls
(``torchsim.mrf_sim``, ``MRFSimulator``, ``FSESimulator``) on small seeded
cases, and records, per case:

* the packed buffers the reference hands its kernel (tissue and the nine event
  buffers), captured at ``_run_packed`` / ``_run_packed_jvp`` /
  ``_run_packed_vjp`` (``src/torchsim/sequence/_accelerators.py:3262, 3933,
  3452``) together with the real-subspace verdict and the raw output planes;
* the public outputs: signal, Jacobian, and gradients of a loss.

The fixtures are what pins the oracle (``oracle/``) and this package's event
builders to the reference. Nothing at test time reads the reference.
"""

from __future__ import annotations

import os
import shutil
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent


def _import_reference(root: Path):
    subprocess.run(["bash", str(REPO / "oracle" / "build_ref.sh"), str(root)], check=True)
    built = sorted((REPO / "oracle" / "_ref").glob("_epg_cpu*.so"))
    if not built:
        raise SystemExit("reference CPU kernel did not build")
    scratch = Path(tempfile.mkdtemp(prefix="torchsim_ref_"))
    shutil.copytree(root / "src" / "torchsim", scratch / "torchsim")
    shutil.copy(built[-1], scratch / "torchsim")
    sys.path.insert(0, str(scratch))
    import torchsim  # noqa: PLC0415

    return torchsim


class _Recorder:
    """Wraps the three packed-run routes and keeps what they were given."""

    def __init__(self, accelerators) -> None:
        self.calls: list[dict] = []
        self.acc = accelerators
        self._orig = {}
        self.verdicts: list = []
        for name in ("_auto_real_axis", "_auto_real_axis_adjoint"):
            self._orig[name] = getattr(accelerators, name)
            setattr(accelerators, name, self._verdict(name))
        for name in ("_run_packed", "_run_packed_jvp", "_run_packed_vjp", "_run_packed_vjp_jvp"):
            self._orig[name] = getattr(accelerators, name)
            setattr(accelerators, name, self._wrap(name))

    def _wrap(self, name):
        original = self._orig[name]

        def wrapped(*args, **kwargs):
            result = original(*args, **kwargs)
            self.calls.append({"route": name, "args": args, "kwargs": kwargs, "result": result})
            return result

        return wrapped

    def _verdict(self, name):
        original = self._orig[name]

        def wrapped(*args, **kwargs):
            result = original(*args, **kwargs)
            self.verdicts.append(result)
            return result

        return wrapped

    def axis(self, call: dict) -> int:
        """The real-subspace verdict a forward call ran under (-1: complex)."""
        args, kwargs = call["args"], call["kwargs"]
        given = args[5] if len(args) > 5 else kwargs.get("real_axis")
        if given is None and self.verdicts:
            given = self.verdicts[0]
        return -1 if given is None else int(given)

    def clear(self) -> None:
        self.calls.clear()
        self.verdicts.clear()


def _np(value):
    import torch

    if torch.is_tensor(value):
        value = value.detach().cpu()
        if value.is_complex():
            return value.numpy().astype(np.complex64 if value.dtype == torch.complex64 else np.complex128)
        return value.numpy()
    return np.asarray(value)


EVENT_NAMES = (
    "duration", "kind", "flip", "phase", "action", "output_index",
    "shim_index", "saturation", "rf_frequency_hz",
)
TISSUE_NAMES = (
    "t1_ms", "t2_ms", "m0", "b1", "b1_phase_rad", "b0_hz", "inversion_efficiency",
    "diffusion_um2_per_ms", "velocity_m_per_s", "bound_fraction", "bound_exchange_hz",
    "t1_bound_ms", "pool_b_fraction", "pool_b_exchange_hz", "t1_pool_b_ms",
    "t2_pool_b_ms", "pool_b_shift_hz",
)


def _packed(call: dict, prefix: str) -> dict:
    args = call["args"]
    tissue, events = args[0], args[1]
    out = {}
    for name, value in zip(TISSUE_NAMES, tissue, strict=True):
        out[f"{prefix}tissue_{name}"] = _np(value)
    for name, value in zip(EVENT_NAMES, events, strict=True):
        out[f"{prefix}event_{name}"] = _np(value)
    return out


def mrf_schedule() -> np.ndarray:
    return np.concatenate(
        [np.linspace(5, 60, 300), np.linspace(60, 2, 300), np.full(280, 2.0)]
    ).astype(np.float32)


def draw_tissue(rng: np.random.Generator, n: int):
    t1 = np.exp(rng.uniform(np.log(100), np.log(3000), n)).astype(np.float32)
    t2 = np.exp(rng.uniform(np.log(10), np.log(300), n)).astype(np.float32)
    t2 = np.minimum(t2, np.float32(0.999) * t1).astype(np.float32)
    b1 = rng.uniform(0.8, 1.2, n).astype(np.float32)
    return t1, t2, b1


def case_mrf880(ts, rec) -> dict:
    import torch

    rng = np.random.default_rng(0)
    t1, t2, b1 = draw_tissue(rng, 8)
    flip = mrf_schedule()
    rec.clear()
    sig = ts.mrf_sim(torch.from_numpy(flip), 10.0, torch.from_numpy(t1), torch.from_numpy(t2),
                     B1=torch.from_numpy(b1), states=10)
    fwd = [c for c in rec.calls if c["route"] == "_run_packed"][0]
    out = {"flip_deg": flip, "tr_ms": np.float32(10.0), "t1": t1, "t2": t2, "b1": b1,
           "states": np.int64(10), "signal": _np(sig)}
    out.update(_packed(fwd, ""))
    out["real_axis"] = np.int64(rec.axis(fwd))
    out["raw_forward"] = _np(fwd["result"])
    rec.clear()
    sig2, jac = ts.mrf_sim(torch.from_numpy(flip), 10.0, torch.from_numpy(t1), torch.from_numpy(t2),
                           B1=torch.from_numpy(b1), states=10, diff=("T1", "T2", "B1", "M0"))
    out["signal_jac"] = _np(sig2)
    out["jacobian"] = _np(jac)
    out["jacobian_names"] = np.array(["T1", "T2", "B1", "M0"])
    return out


def case_mrf_prep(ts, rec) -> dict:
    import torch

    rng = np.random.default_rng(1)
    n = 5
    t1, t2, b1 = draw_tissue(rng, n)
    m0 = rng.uniform(0.5, 1.5, n).astype(np.float32)
    inv = rng.uniform(0.85, 1.0, n).astype(np.float32)
    flip = rng.uniform(5, 70, 60).astype(np.float32)
    tr = rng.uniform(8, 15, 60).astype(np.float32)
    kw = dict(B1=torch.from_numpy(b1), M0=torch.from_numpy(m0), inv_efficiency=torch.from_numpy(inv),
              TI=20.0, states=7, nreps=2)
    rec.clear()
    sig = ts.mrf_sim(torch.from_numpy(flip), torch.from_numpy(tr), torch.from_numpy(t1),
                     torch.from_numpy(t2), **kw)
    fwd = [c for c in rec.calls if c["route"] == "_run_packed"][0]
    out = {"flip_deg": flip, "tr_ms": tr, "t1": t1, "t2": t2, "b1": b1, "m0": m0, "inv": inv,
           "ti_ms": np.float32(20.0), "nreps": np.int64(2), "states": np.int64(7),
           "signal": _np(sig)}
    out.update(_packed(fwd, ""))
    out["real_axis"] = np.int64(rec.axis(fwd))
    out["raw_forward"] = _np(fwd["result"])
    names = ("T1", "T2", "B1", "M0", "inv_efficiency")
    _, jac = ts.mrf_sim(torch.from_numpy(flip), torch.from_numpy(tr), torch.from_numpy(t1),
                        torch.from_numpy(t2), diff=names, **kw)
    out["jacobian"] = _np(jac)
    out["jacobian_names"] = np.array(names)
    return out


def case_fse(ts, rec) -> dict:
    import torch
    from torchsim.simulators import FSESimulator

    rng = np.random.default_rng(2)
    n, etl = 6, 12
    t1 = rng.uniform(300, 3000, n).astype(np.float32)
    t2 = rng.uniform(10, 300, n).astype(np.float32)
    b1 = rng.uniform(0.7, 1.3, n).astype(np.float32)
    flip = rng.uniform(100, 180, etl).astype(np.float32)
    esp = 8.0
    sim = FSESimulator(flip=torch.from_numpy(flip), ESP=esp, phases=90.0, states=2 * etl)
    rec.clear()
    sig = sim.simulate(T1=torch.from_numpy(t1), T2=torch.from_numpy(t2), B1=torch.from_numpy(b1))
    fwd = [c for c in rec.calls if c["route"] == "_run_packed"][0]
    out = {"flip_deg": flip, "esp_ms": np.float32(esp), "t1": t1, "t2": t2, "b1": b1,
           "states": np.int64(2 * etl), "signal": _np(sig)}
    out.update(_packed(fwd, ""))
    out["real_axis"] = np.int64(rec.axis(fwd))
    out["raw_forward"] = _np(fwd["result"])
    names = ("T1", "T2", "B1")
    _, jac = sim.jacobian(names, T1=torch.from_numpy(t1), T2=torch.from_numpy(t2), B1=torch.from_numpy(b1))
    out["jacobian"] = _np(jac)
    out["jacobian_names"] = np.array(names)
    return out


def case_fse_phase0(ts, rec) -> dict:
    """Default-phase CPMG (refocusing at 0 deg, excitation at 90 deg): the
    reference leaves the real subspace and runs its complex kernel."""
    import torch
    from torchsim.simulators import FSESimulator

    rng = np.random.default_rng(5)
    n, etl = 6, 10
    t1 = rng.uniform(300, 3000, n).astype(np.float32)
    t2 = rng.uniform(10, 300, n).astype(np.float32)
    b1 = rng.uniform(0.7, 1.3, n).astype(np.float32)
    flip = rng.uniform(100, 180, etl).astype(np.float32)
    esp = 9.0
    sim = FSESimulator(flip=torch.from_numpy(flip), ESP=esp, states=2 * etl)
    rec.clear()
    sig = sim.simulate(T1=torch.from_numpy(t1), T2=torch.from_numpy(t2), B1=torch.from_numpy(b1))
    fwd = [c for c in rec.calls if c["route"] == "_run_packed"][0]
    out = {"flip_deg": flip, "esp_ms": np.float32(esp), "t1": t1, "t2": t2, "b1": b1,
           "states": np.int64(2 * etl), "signal": _np(sig)}
    out.update(_packed(fwd, ""))
    out["real_axis"] = np.int64(rec.axis(fwd))
    out["raw_forward"] = _np(fwd["result"])
    names = ("T1", "T2", "B1")
    _, jac = sim.jacobian(names, T1=torch.from_numpy(t1), T2=torch.from_numpy(t2),
                          B1=torch.from_numpy(b1))
    out["jacobian"] = _np(jac)
    out["jacobian_names"] = np.array(names)
    return out


def case_mrf_offaxis(ts, rec) -> dict:
    """MRF with off-resonance (B0) and a transmit phase (B1phase) per voxel:
    the complex kernel with phase turns in the relaxation and the pulses."""
    import torch
    from torchsim.simulators import MRFSimulator

    rng = np.random.default_rng(6)
    n, pulses = 8, 60
    t1, t2, b1 = draw_tissue(rng, n)
    b0 = rng.uniform(-40, 40, n).astype(np.float32)
    b1p = rng.uniform(-0.5, 0.5, n).astype(np.float32)
    m0 = rng.uniform(0.5, 1.5, n).astype(np.float32)
    flip = rng.uniform(5, 70, pulses).astype(np.float32)
    tr = rng.uniform(8, 15, pulses).astype(np.float32)
    sim = MRFSimulator(flip=torch.from_numpy(flip), TR=torch.from_numpy(tr), TI=15.0, states=12)
    rec.clear()
    sig = sim.simulate(T1=torch.from_numpy(t1), T2=torch.from_numpy(t2), B1=torch.from_numpy(b1),
                       B0=torch.from_numpy(b0), B1phase=torch.from_numpy(b1p),
                       M0=torch.from_numpy(m0))
    fwd = [c for c in rec.calls if c["route"] == "_run_packed"][0]
    out = {"flip_deg": flip, "tr_ms": tr, "ti_ms": np.float32(15.0), "t1": t1, "t2": t2,
           "b1": b1, "b0": b0, "b1_phase": b1p, "m0": m0, "states": np.int64(12),
           "signal": _np(sig)}
    out.update(_packed(fwd, ""))
    out["real_axis"] = np.int64(rec.axis(fwd))
    out["raw_forward"] = _np(fwd["result"])
    names = ("T1", "T2", "B1", "M0")
    _, jac = sim.jacobian(names, T1=torch.from_numpy(t1), T2=torch.from_numpy(t2),
                          B1=torch.from_numpy(b1), B0=torch.from_numpy(b0),
                          B1phase=torch.from_numpy(b1p), M0=torch.from_numpy(m0))
    out["jacobian"] = _np(jac)
    out["jacobian_names"] = np.array(names)
    return out


def case_complex_jvp(ts, rec) -> dict:
    """Forward-mode tangents on the complex path, as the reference's own
    _run_packed_jvp computes them (its complex simulate_jvp_range): an MRF
    train with RF phases, per-voxel B0, B1phase, M0 and inversion efficiency,
    differentiated along each tissue property the public Jacobian offers
    (one call each) and along one direction in flip, TR and phase at once.
    Each recorded call keeps its packed buffers, tangents and result."""
    import torch
    from torchsim.simulators import MRFSimulator

    rng = np.random.default_rng(12)
    n, pulses = 6, 50
    t1, t2, b1 = draw_tissue(rng, n)
    b0 = rng.uniform(-40, 40, n).astype(np.float32)
    b1p = rng.uniform(-0.5, 0.5, n).astype(np.float32)
    m0 = rng.uniform(0.5, 1.5, n).astype(np.float32)
    inv = rng.uniform(0.85, 1.0, n).astype(np.float32)
    flip = rng.uniform(5, 70, pulses).astype(np.float32)
    tr = rng.uniform(8, 15, pulses).astype(np.float32)
    phases = rng.uniform(-40, 40, pulses).astype(np.float32)
    values = {"T1": torch.from_numpy(t1), "T2": torch.from_numpy(t2),
              "B1": torch.from_numpy(b1), "B0": torch.from_numpy(b0),
              "B1phase": torch.from_numpy(b1p), "M0": torch.from_numpy(m0),
              "inv_efficiency": torch.from_numpy(inv)}
    sim = MRFSimulator(TI=15.0, states=12)
    protocol = {"flip": torch.from_numpy(flip), "TR": torch.from_numpy(tr),
                "phases": torch.from_numpy(phases)}
    rec.clear()
    names = ("T1", "T2", "B1", "M0", "inv_efficiency", "B0", "B1phase")
    _, jac = sim.jacobian(names, **protocol, **values)
    directions = {"flip": rng.standard_normal(pulses).astype(np.float32),
                  "TR": rng.standard_normal(pulses).astype(np.float32) * 0.5,
                  "phases": rng.standard_normal(pulses).astype(np.float32) * 5}

    def played(f, r, p):
        return sim.simulate(flip=f, TR=r, phases=p, **values)

    _, along = torch.func.jvp(
        played, (protocol["flip"], protocol["TR"], protocol["phases"]),
        tuple(torch.from_numpy(directions[k]) for k in ("flip", "TR", "phases")))
    calls = [c for c in rec.calls if c["route"] == "_run_packed_jvp"]
    out = {"jacobian": _np(jac), "jacobian_names": np.array(names), "along": _np(along),
           "states": np.int64(12), "calls": np.int64(len(calls)), "flip_deg": flip, "tr_ms": tr,
           "phases_deg": phases, "ti_ms": np.float32(15.0), "t1": t1, "t2": t2, "b1": b1,
           "b0": b0, "b1_phase": b1p, "m0": m0, "inv": inv,
           **{f"direction_{k}": v for k, v in directions.items()}}
    for k, call in enumerate(calls):
        args = call["args"]
        out.update(_packed(call, f"c{k}_"))
        for j, value in enumerate(args[2]):
            out[f"c{k}_tissue_tangent_{j}"] = _np(value)
        for j, value in enumerate(args[3]):
            out[f"c{k}_event_tangent_{j}"] = _np(value)
        axis = args[7] if len(args) > 7 else call["kwargs"].get("real_axis")
        out[f"c{k}_real_axis"] = np.int64(-1 if axis is None else axis)
        out[f"c{k}_result"] = _np(call["result"])
    return out


def case_adjoint(ts, rec) -> dict:
    import torch
    from torchsim.simulators import MRFSimulator

    rng = np.random.default_rng(3)
    n, pulses = 4, 40
    t1, t2, b1 = draw_tissue(rng, n)
    flip = rng.uniform(5, 70, pulses).astype(np.float32)
    tr = rng.uniform(8, 15, pulses).astype(np.float32)
    target_flip = rng.uniform(5, 70, pulses).astype(np.float32)
    target_tr = rng.uniform(8, 15, pulses).astype(np.float32)
    tissue = dict(T1=torch.from_numpy(t1), T2=torch.from_numpy(t2), B1=torch.from_numpy(b1))
    with torch.no_grad():
        target = MRFSimulator(flip=torch.from_numpy(target_flip), TR=torch.from_numpy(target_tr),
                              states=8).simulate(**tissue)
    theta = torch.from_numpy(flip).clone().requires_grad_(True)
    tau = torch.from_numpy(tr).clone().requires_grad_(True)
    t1t = torch.from_numpy(t1).clone().requires_grad_(True)
    t2t = torch.from_numpy(t2).clone().requires_grad_(True)
    b1t = torch.from_numpy(b1).clone().requires_grad_(True)
    rec.clear()
    sig = MRFSimulator(flip=theta, TR=tau, states=8).simulate(T1=t1t, T2=t2t, B1=b1t)
    loss = (sig - target).abs().square().sum()
    loss.backward()
    out = {"flip_deg": flip, "tr_ms": tr, "t1": t1, "t2": t2, "b1": b1, "states": np.int64(8),
           "target": _np(target), "signal": _np(sig), "loss": _np(loss),
           "grad_flip_deg": _np(theta.grad), "grad_tr_ms": _np(tau.grad),
           "grad_t1": _np(t1t.grad), "grad_t2": _np(t2t.grad), "grad_b1": _np(b1t.grad)}
    out["adjoint_verdicts"] = np.array([-1 if v is None else int(v) for v in rec.verdicts])
    vjp = [c for c in rec.calls if c["route"] == "_run_packed_vjp"]
    if vjp:
        call = vjp[0]
        out.update(_packed(call, "vjp_"))
        out["vjp_seed"] = _np(call["args"][2])
        names = (*TISSUE_NAMES, "duration", "flip", "phase")
        for name, value in zip(names, call["result"], strict=True):
            if value is not None:
                out[f"vjp_grad_{name}"] = _np(value)
    return out


def _vjp_record(rec, prefix: str) -> dict:
    """The packed buffers, seed and gradients of the first recorded
    ``_run_packed_vjp`` call."""
    out = {}
    vjp = [c for c in rec.calls if c["route"] == "_run_packed_vjp"]
    call = vjp[0]
    out.update(_packed(call, prefix))
    out[prefix + "seed"] = _np(call["args"][2])
    names = (*TISSUE_NAMES, "duration", "flip", "phase")
    for name, value in zip(names, call["result"], strict=True):
        if value is not None:
            out[f"{prefix}grad_{name}"] = _np(value)
    return out


def case_complex_adjoint(ts, rec) -> dict:
    """Gradients on the complex path: an off-axis MRF (B0, B1phase, M0 maps)
    with every tissue map, flip and TR a leaf, and a default-phase CPMG with
    its refocusing flips and tissue as leaves; loss sum |s - target|^2."""
    import torch
    from torchsim.simulators import FSESimulator, MRFSimulator

    rng = np.random.default_rng(8)
    n, pulses = 5, 30
    t1, t2, b1 = draw_tissue(rng, n)
    b0 = rng.uniform(-40, 40, n).astype(np.float32)
    b1p = rng.uniform(-0.5, 0.5, n).astype(np.float32)
    m0 = rng.uniform(0.5, 1.5, n).astype(np.float32)
    flip = rng.uniform(5, 70, pulses).astype(np.float32)
    tr = rng.uniform(8, 15, pulses).astype(np.float32)
    target = (rng.standard_normal((n, pulses)) + 1j * rng.standard_normal((n, pulses)))
    target = (0.05 * target).astype(np.complex64)
    leaves = {k: torch.from_numpy(v).clone().requires_grad_(True) for k, v in
              (("T1", t1), ("T2", t2), ("B1", b1), ("B0", b0), ("B1phase", b1p), ("M0", m0))}
    theta = torch.from_numpy(flip).clone().requires_grad_(True)
    tau = torch.from_numpy(tr).clone().requires_grad_(True)
    rec.clear()
    sig = MRFSimulator(flip=theta, TR=tau, TI=15.0, states=10).simulate(**leaves)
    loss = (sig - torch.from_numpy(target)).abs().square().sum()
    loss.backward()
    out = {"mrf_flip_deg": flip, "mrf_tr_ms": tr, "mrf_t1": t1, "mrf_t2": t2, "mrf_b1": b1,
           "mrf_b0": b0, "mrf_b1_phase": b1p, "mrf_m0": m0, "mrf_states": np.int64(10),
           "mrf_target": target, "mrf_signal": _np(sig), "mrf_loss": _np(loss),
           "mrf_grad_flip_deg": _np(theta.grad), "mrf_grad_tr_ms": _np(tau.grad)}
    for k, v in leaves.items():
        out[f"mrf_grad_{k}"] = _np(v.grad)
    out.update(_vjp_record(rec, "mrf_vjp_"))
    # Default-phase CPMG.
    etl = 8
    t1f = rng.uniform(300, 3000, 4).astype(np.float32)
    t2f = rng.uniform(10, 300, 4).astype(np.float32)
    b1f = rng.uniform(0.7, 1.3, 4).astype(np.float32)
    refoc = rng.uniform(100, 180, etl).astype(np.float32)
    ftarget = (0.05 * rng.standard_normal((4, etl))).astype(np.complex64)
    fleaves = {k: torch.from_numpy(v).clone().requires_grad_(True) for k, v in
               (("T1", t1f), ("T2", t2f), ("B1", b1f))}
    phi = torch.from_numpy(refoc).clone().requires_grad_(True)
    rec.clear()
    fsig = FSESimulator(flip=phi, ESP=9.0, states=2 * etl).simulate(**fleaves)
    floss = (fsig - torch.from_numpy(ftarget)).abs().square().sum()
    floss.backward()
    out.update({"fse_flip_deg": refoc, "fse_esp_ms": np.float32(9.0), "fse_t1": t1f,
                "fse_t2": t2f, "fse_b1": b1f, "fse_states": np.int64(2 * etl),
                "fse_target": ftarget, "fse_signal": _np(fsig), "fse_loss": _np(floss),
                "fse_grad_flip_deg": _np(phi.grad)})
    for k, v in fleaves.items():
        out[f"fse_grad_{k}"] = _np(v.grad)
    out.update(_vjp_record(rec, "fse_vjp_"))
    return out


def case_second(ts, rec) -> dict:
    """Second order. A Cramer-Rao cost of the (T1, T2) Jacobian differentiated
    with respect to the flip angles and TRs: the reference's design route
    (``_NativeEpgJvp.backward`` -> ``_run_packed_vjp_jvp``, one call per
    Jacobian column), and one direct forward-over-reverse call with a general
    direction (every tissue property, duration and flip) and a random seed."""
    import torch
    from torchsim.optim import crlb
    from torchsim.simulators import MRFSimulator

    rng = np.random.default_rng(5)
    n, pulses = 3, 30
    t1, t2, b1 = draw_tissue(rng, n)
    m0 = rng.uniform(0.5, 1.5, n).astype(np.float32)
    flip = rng.uniform(5, 70, pulses).astype(np.float32)
    tr = rng.uniform(8, 15, pulses).astype(np.float32)
    theta = torch.from_numpy(flip).clone().requires_grad_(True)
    tau = torch.from_numpy(tr).clone().requires_grad_(True)
    tissue = dict(T1=torch.from_numpy(t1), T2=torch.from_numpy(t2), B1=torch.from_numpy(b1),
                  M0=torch.from_numpy(m0))
    rec.clear()
    sig, jac = MRFSimulator(flip=theta, TR=tau, states=8).jacobian(("T1", "T2"), **tissue)
    scale = torch.stack((tissue["T1"], tissue["T2"]), dim=-1)
    loss = (crlb(jac) / scale.square()).sum()
    loss.backward()
    out = {"flip_deg": flip, "tr_ms": tr, "t1": t1, "t2": t2, "b1": b1, "m0": m0,
           "states": np.int64(8), "signal": _np(sig), "jacobian": _np(jac), "loss": _np(loss),
           "grad_flip_deg": _np(theta.grad), "grad_tr_ms": _np(tau.grad)}
    calls = [c for c in rec.calls if c["route"] == "_run_packed_vjp_jvp"]
    names = (*TISSUE_NAMES, "duration", "flip", "phase")
    out["design_calls"] = np.int64(len(calls))
    for k, call in enumerate(calls):
        args = call["args"]
        out.update(_packed(call, f"design{k}_"))
        for name, value in zip(names, args[2], strict=True):
            out[f"design{k}_tangent_{name}"] = _np(value)
        out[f"design{k}_seed"] = _np(args[3])
        curvature, values = call["result"]
        for name, value in zip(names, curvature, strict=False):
            out[f"design{k}_curvature_{name}"] = _np(value)
        for name, value in zip(names, values, strict=False):
            out[f"design{k}_value_{name}"] = _np(value)
    # The direct call: the packed buffers of a plain forward of the same case.
    rec.clear()
    with torch.no_grad():
        MRFSimulator(flip=torch.from_numpy(flip), TR=torch.from_numpy(tr), states=8).simulate(
            **tissue, inv_efficiency=torch.from_numpy(rng.uniform(0.8, 1.0, n).astype(np.float32)))
    fwd = [c for c in rec.calls if c["route"] == "_run_packed"][0]
    packed_tissue, events = fwd["args"][0], fwd["args"][1]
    output_count = int(fwd["result"].shape[-1])
    gen = torch.Generator().manual_seed(6)
    tangents = []
    for name, value in zip(names, (*packed_tissue, events[0], events[2], events[3]), strict=True):
        if name in ("t1_ms", "t2_ms", "m0", "b1", "inversion_efficiency", "duration", "flip"):
            t = torch.randn(value.shape, generator=gen, dtype=value.dtype)
            t = t * (100.0 if name in ("t1_ms", "t2_ms") else 1e-3 if name == "duration" else 0.1)
        else:
            t = torch.zeros_like(value)
        tangents.append(t)
    seed = torch.randn((n, output_count), generator=gen, dtype=torch.complex64)
    rec.clear()
    curvature, values = _accelerators_of(ts)._run_packed_vjp_jvp(
        tuple(packed_tissue), tuple(events), tuple(tangents), seed, state_count=8,
        output_count=output_count, threads=1, real_axis=1)
    out.update(_packed(fwd, "direct_"))
    for name, value in zip(names, tangents, strict=True):
        out[f"direct_tangent_{name}"] = _np(value)
    out["direct_seed"] = _np(seed)
    for name, value in zip(names, curvature, strict=False):
        out[f"direct_curvature_{name}"] = _np(value)
    for name, value in zip(names, values, strict=False):
        out[f"direct_value_{name}"] = _np(value)
    return out


def case_double_backward(ts, rec) -> dict:
    """Reverse over reverse through the public simulator: the gradient of
    <directions, d<seed, s>/d(inputs)> with respect to the inputs and the
    seed (the reference's _NativeEpg backward differentiated once more)."""
    import torch
    from torchsim.simulators import MRFSimulator

    rng = np.random.default_rng(9)
    n, pulses = 4, 25
    t1, t2, b1 = draw_tissue(rng, n)
    m0 = rng.uniform(0.5, 1.5, n).astype(np.float32)
    flip = rng.uniform(5, 70, pulses).astype(np.float32)
    tr = rng.uniform(8, 15, pulses).astype(np.float32)
    leaves = {k: torch.from_numpy(v).clone().requires_grad_(True) for k, v in
              (("T1", t1), ("T2", t2), ("B1", b1), ("M0", m0))}
    theta = torch.from_numpy(flip).clone().requires_grad_(True)
    tau = torch.from_numpy(tr).clone().requires_grad_(True)
    sig = MRFSimulator(flip=theta, TR=tau, states=8).simulate(**leaves)
    gen = torch.Generator().manual_seed(4)
    seed = torch.randn(sig.shape, generator=gen, dtype=torch.complex64).requires_grad_(True)
    inputs = (theta, tau, *leaves.values())
    grads = torch.autograd.grad(sig, inputs, seed, create_graph=True)
    directions = [torch.randn(g.shape, generator=gen) for g in grads]
    contraction = sum((g * d).sum() for g, d in zip(grads, directions, strict=True))
    second = torch.autograd.grad(contraction, (*inputs, seed))
    out = {"flip_deg": flip, "tr_ms": tr, "t1": t1, "t2": t2, "b1": b1, "m0": m0,
           "states": np.int64(8), "seed": _np(seed), "contraction": _np(contraction)}
    names = ("flip_deg", "tr_ms", "T1", "T2", "B1", "M0")
    for name, g, d, h in zip(names, grads, directions, second[:-1], strict=True):
        out[f"grad_{name}"] = _np(g)
        out[f"direction_{name}"] = _np(d)
        out[f"second_{name}"] = _np(h)
    out["second_seed"] = _np(second[-1])
    return out


def case_grouping(ts, rec) -> dict:
    """The reference's group matching (estimators/_grouped.py) on a
    deterministic family of complex decays: the greedy clustering into 24
    groups, the representatives, the surviving groups of noisy signals at
    three thresholds and the top-3 grouped match."""
    import torch
    from torchsim.estimators._grouped import Grouping, match_in_groups

    t = torch.linspace(0.01, 3.0, 60, dtype=torch.float64)
    r1 = torch.linspace(0.3, 5.0, 20, dtype=torch.float64)
    r2 = torch.linspace(1.0, 30.0, 25, dtype=torch.float64)
    g1, g2 = torch.meshgrid(r1, r2, indexing="ij")
    atoms = (1 - 2 * torch.exp(-t * g1.reshape(-1, 1))) * torch.exp(-t * g2.reshape(-1, 1) / 10)
    atoms = atoms.to(torch.complex64) * (1 + 0.5j)
    grouping = Grouping.fit(atoms, 24)
    gen = torch.Generator().manual_seed(7)
    picked = atoms[::13]
    noise = torch.randn(picked.shape, generator=gen, dtype=torch.complex64)
    signals = picked + 0.01 * float(atoms.abs().max()) * noise
    unit = signals / torch.linalg.vector_norm(signals, dim=-1, keepdim=True)
    out = {"atoms": _np(atoms), "signals": _np(signals),
           "members": np.concatenate([_np(m) for m in grouping.members]),
           "sizes": np.array(grouping.sizes, np.int64),
           "representative": _np(grouping.representative),
           "condition": np.float64(grouping.condition)}
    for prune in (0.0, 5e-3, 0.2):
        out[f"survivors_{prune:g}"] = _np(grouping.survivors(unit, prune))
    indices, scores = match_in_groups(unit, grouping, 3, 5e-3)
    out["match_indices"] = _np(indices)
    out["match_scores"] = _np(scores)
    return out


def case_design_loop(ts, rec) -> dict:
    """The reference's design layer on a pure-torch cost (optim/_design.py):
    crlb of real and complex Jacobians (and the infinite answer where the
    Fisher matrix is singular), and SequenceDesign.minimize with two bounded
    parameter vectors, one with per-element limits, for 25 Adam steps."""
    import torch
    from torchsim.optim import Bounded, SequenceDesign, crlb

    gen = torch.Generator().manual_seed(3)
    real = torch.randn((5, 3, 40), generator=gen)
    cplx = torch.randn((5, 3, 40), generator=gen, dtype=torch.complex64)
    singular = real.clone()
    singular[2, 1] = singular[2, 0]
    flip0 = torch.linspace(10.0, 60.0, 12)
    tr0 = torch.full((12,), 11.0)
    target = torch.rand(12, generator=gen) * 0.8 + 0.1
    upper = torch.linspace(40.0, 70.0, 12)

    def cost(flip, tr):
        return ((torch.sin(torch.deg2rad(flip)) - target) ** 2).sum() + 1e-3 * (tr - 9.0).square().sum()

    design = SequenceDesign(cost, flip=Bounded(flip0, 5.0, upper), tr=Bounded(tr0, 8.0, 15.0))
    result = design.minimize(iterations=25, learning_rate=0.05)
    return {"real": _np(real), "complex": _np(cplx), "singular": _np(singular),
            "crlb_real": _np(crlb(real, noise_variance=0.5)),
            "crlb_complex": _np(crlb(cplx, noise_variance=0.5)),
            "crlb_singular": _np(crlb(singular, singular="infinite")),
            "flip0": _np(flip0), "tr0": _np(tr0), "target": _np(target), "upper": _np(upper),
            "loss": _np(result.loss), "flip": _np(result.parameters["flip"]),
            "tr": _np(result.parameters["tr"])}


def case_bounds(ts, rec) -> dict:
    """The reference's variable transforms (_bounds.py): to_free of values
    inside two-sided, lower-only, upper-only and absent bounds, including
    values at the very edges (clamped), and to_natural back."""
    import torch
    from torchsim._bounds import to_free, to_natural

    bounds = {"T1": (50.0, 5000.0), "T2": (2.0, None), "M0": (None, 5.0)}
    names = ("T1", "T2", "M0", "B1")
    gen = torch.Generator().manual_seed(5)
    natural = torch.stack([
        torch.cat([50.0 + 4950.0 * torch.rand(60, generator=gen, dtype=torch.float64),
                   torch.tensor([50.0, 5000.0, 50.0 + 1e-9], dtype=torch.float64)]),
        torch.cat([2.0 + torch.exp(6 * torch.randn(60, generator=gen, dtype=torch.float64)),
                   torch.tensor([2.0, 2.0 + 1e-9, 1e6], dtype=torch.float64)]),
        torch.cat([5.0 - torch.exp(3 * torch.randn(60, generator=gen, dtype=torch.float64)),
                   torch.tensor([5.0, -1e3, 5.0 - 1e-9], dtype=torch.float64)]),
        torch.randn(63, generator=gen, dtype=torch.float64),
    ], dim=-1)
    free = to_free(natural, bounds, names)
    return {"natural": _np(natural), "free": _np(free),
            "back": _np(to_natural(free, bounds, names))}


def _accelerators_of(ts):
    from torchsim.sequence import _accelerators

    return _accelerators


def case_gn(ts, rec) -> dict:
    """The reference's NonlinearLeastSquares (Levenberg-Marquardt, default
    loop: TrustRegion, direct, 20 iterations) on noisy MRF signals."""
    import torch
    from torchsim import NonlinearLeastSquares
    from torchsim.simulators import MRFSimulator

    rng = np.random.default_rng(4)
    n, v = 120, 16
    flip = np.concatenate([np.linspace(5, 60, 60), np.linspace(60, 2, 60)]).astype(np.float32)
    t1, t2, b1 = draw_tissue(rng, v)
    m0 = rng.uniform(0.5, 1.5, v).astype(np.float32)
    sim = MRFSimulator(flip=torch.from_numpy(flip), TR=10.0, states=10)
    with torch.no_grad():
        sig = sim.simulate(T1=torch.from_numpy(t1), T2=torch.from_numpy(t2),
                           B1=torch.from_numpy(b1), M0=torch.from_numpy(m0))
    sigma = float(sig.abs().mean()) / 50.0
    noise = (rng.standard_normal(sig.shape) + 1j * rng.standard_normal(sig.shape)) * sigma
    y = (sig.numpy() + noise).astype(np.complex64)
    bounds = {"T1": (50.0, 5000.0), "T2": (2.0, 1000.0), "M0": (0.0, 5.0)}
    est = NonlinearLeastSquares(sim, bounds=bounds)
    est.fit(T1=(100.0, 3000.0), T2=(10.0, 300.0), M0=(0.5, 1.5), known={"B1": (0.8, 1.2)}, seed=0)
    maps = est.map(torch.from_numpy(y), known={"B1": torch.from_numpy(b1)})
    return {"flip_deg": flip, "tr_ms": np.float32(10.0), "states": np.int64(10), "t1": t1,
            "t2": t2, "b1": b1, "m0": m0, "measured": y, "start": est._start.numpy(),
            "bounds": np.array([bounds[k] for k in ("T1", "T2", "M0")], np.float64),
            "map_t1": maps["T1"].numpy(), "map_t2": maps["T2"].numpy(),
            "map_m0": maps["M0"].numpy(), "iterations": np.int64(est.iterations),
            "unconverged": np.int64(est.unconverged)}


def case_gn_slice(ts, rec) -> dict:
    """The reference's NonlinearLeastSquares on a 4,096-voxel slice (the
    mapping workload's request size), B1 known. The measured signals are not
    stored: they are the reference's noise-free signal, which the oracle's
    FP32 port reproduces bit for bit from the stored tissue, plus complex
    Gaussian noise drawn from `noise_seed` and scaled by the stored `sigma`;
    every 64th row of them is kept to check the regeneration."""
    import torch
    from torchsim import NonlinearLeastSquares
    from torchsim.simulators import MRFSimulator

    rng = np.random.default_rng(9)
    v = 4096
    flip = np.concatenate([np.linspace(5, 60, 60), np.linspace(60, 2, 60)]).astype(np.float32)
    t1, t2, b1 = draw_tissue(rng, v)
    m0 = rng.uniform(0.5, 1.5, v).astype(np.float32)
    sim = MRFSimulator(flip=torch.from_numpy(flip), TR=10.0, states=10)
    with torch.no_grad():
        sig = sim.simulate(T1=torch.from_numpy(t1), T2=torch.from_numpy(t2),
                           B1=torch.from_numpy(b1), M0=torch.from_numpy(m0))
    sigma = float(sig.abs().mean()) / 50.0
    noise_seed = 90
    nrng = np.random.default_rng(noise_seed)
    noise = (nrng.standard_normal(sig.shape) + 1j * nrng.standard_normal(sig.shape)) * sigma
    y = (sig.numpy() + noise).astype(np.complex64)
    bounds = {"T1": (50.0, 5000.0), "T2": (2.0, 1000.0), "M0": (0.0, 5.0)}
    est = NonlinearLeastSquares(sim, bounds=bounds)
    est.fit(T1=(100.0, 3000.0), T2=(10.0, 300.0), M0=(0.5, 1.5), known={"B1": (0.8, 1.2)}, seed=0)
    maps = est.map(torch.from_numpy(y), known={"B1": torch.from_numpy(b1)})
    return {"flip_deg": flip, "tr_ms": np.float32(10.0), "states": np.int64(10), "t1": t1,
            "t2": t2, "b1": b1, "m0": m0, "sigma": np.float64(sigma),
            "noise_seed": np.int64(noise_seed), "measured_every_64th": y[::64],
            "start": est._start.numpy(),
            "bounds": np.array([bounds[k] for k in ("T1", "T2", "M0")], np.float64),
            "map_t1": maps["T1"].numpy(), "map_t2": maps["T2"].numpy(),
            "map_m0": maps["M0"].numpy(), "iterations": np.int64(est.iterations),
            "unconverged": np.int64(est.unconverged)}


CASES = ("mrf880", "mrf_prep", "fse_cpmg", "mrf_adjoint", "gn_mrf", "fse_phase0", "mrf_offaxis",
         "complex_jvp", "gn_slice",
         "mrf_second", "complex_adjoint", "double_backward", "grouping", "design_loop", "bounds")


def main() -> None:
    args = sys.argv[1:]
    root = Path(args[0] if args and args[0] not in CASES
                else os.environ.get("TORCHSIM_REFERENCE", "/root/reference"))
    wanted = [a for a in args if a in CASES] or list(CASES)
    os.environ.setdefault("OMP_NUM_THREADS", "1")
    ts = _import_reference(root)
    import torch

    torch.manual_seed(0)
    from torchsim.sequence import _accelerators

    # Reach for the real-subspace verdict however small the case, as the
    # reference's own tests do (tests/conftest.py:6-17), so the fixtures come
    # from the kernels this package restates.
    _accelerators.detection = lambda kind, device: 0.0
    rec = _Recorder(_accelerators)
    for name, fn in (("mrf880", case_mrf880), ("mrf_prep", case_mrf_prep),
                     ("fse_cpmg", case_fse), ("mrf_adjoint", case_adjoint), ("gn_mrf", case_gn),
                     ("fse_phase0", case_fse_phase0), ("mrf_offaxis", case_mrf_offaxis),
                     ("mrf_second", case_second), ("complex_adjoint", case_complex_adjoint),
                     ("double_backward", case_double_backward), ("grouping", case_grouping),
                     ("design_loop", case_design_loop), ("bounds", case_bounds),
                     ("complex_jvp", case_complex_jvp), ("gn_slice", case_gn_slice)):
        if name not in wanted:
            continue
        data = fn(ts, rec)
        np.savez_compressed(HERE / f"{name}.npz", **data)
        print(f"wrote {name}.npz with {len(data)} arrays")


if __name__ == "__main__":
    main()
