"""Event builders reproduce the reference's packed buffers bit for bit."""

from __future__ import annotations

import numpy as np
import pytest
import torch

from torchsim_gb300.sequence import fse_events, mrf_events

FIELDS = ("duration", "kind", "flip", "phase", "action", "output_index")


def _check(events, d):
    for name in FIELDS:
        ref = d["event_" + name]
        mine = getattr(events, name).reshape(ref.shape)
        assert mine.dtype == ref.dtype, name
        assert np.array_equal(mine, ref), name


def test_mrf880(golden):
    d = golden("mrf880")
    _check(mrf_events(torch.from_numpy(d["flip_deg"]), 10.0), d)


def test_mrf_prepared_repeated(golden):
    d = golden("mrf_prep")
    ev = mrf_events(torch.from_numpy(d["flip_deg"]), torch.from_numpy(d["tr_ms"]),
                    TI_ms=float(d["ti_ms"]), repetitions=int(d["nreps"]))
    _check(ev, d)
    assert ev.outputs == 60


def test_fse_cpmg(golden):
    d = golden("fse_cpmg")
    _check(fse_events(torch.from_numpy(d["flip_deg"]), float(d["esp_ms"]), phases_deg=90.0), d)


def test_adjoint_case_stream(golden):
    d = golden("mrf_adjoint")
    ev = mrf_events(torch.from_numpy(d["flip_deg"]), torch.from_numpy(d["tr_ms"]))
    for name in FIELDS:
        ref = d["vjp_event_" + name]
        assert np.array_equal(getattr(ev, name).reshape(ref.shape), ref), name


def test_real_axis_verdict():
    assert mrf_events(np.float32([10, 20]), 10.0).real_axis() == 1
    assert fse_events(np.float32([180, 120]), 10.0, phases_deg=90.0).real_axis() == 1
    # Default-phase CPMG puts the refocusing off the excitation axis.
    assert fse_events(np.float32([180, 120]), 10.0, phases_deg=0.0).real_axis() == -1
    with pytest.raises(ValueError):
        mrf_events(np.float32([10, 20]), np.float32([1, 2, 3]))


def test_mrf_builder_edges():
    with pytest.raises(ValueError):
        mrf_events(np.float32([]), 10.0)
    one = mrf_events(np.float32([30.0]), 12.0, TI_ms=5.0)
    assert one.events == 5 and one.outputs == 1
    assert np.allclose(one.time_us, [5000.0])
    two = mrf_events(np.float32([30.0, 40.0]), 12.0, repetitions=3)
    assert two.events == 27 and two.outputs == 2
    # The recorded samples are the last playing's: two trains after the first.
    assert np.allclose(two.time_us, [2 * 24000.0, 2 * 24000.0 + 12000.0])
