"""The pulse-program compiler's op shapes for the two sequence families the
sweep kernels run on straight-line paths (host only). An MRF repetition
compiles to one op "relax, rotate, record, one shift after"; a CPMG echo to a
refocusing op "relax, shift, rotate, shift" and a recording op. The kernels
recognise those codes with fixed masks; a compiler change that moved either
family off them would keep the results but lose the fast path, so the codes
are pinned here. Bits (csrc/tsg_internal.h): relax 1, shift before the pulse
bits 1-2, RF bits 3-4 (1 rotate, 2 invert), shift after the pulse bits 5-6,
spoil 7, record 8, shift after the record bits 9-10, spoil 11."""

from __future__ import annotations

import numpy as np

from tests.helpers import mrf_schedule

RELAX, ROTATE, INVERT, RECORD = 1, 1 << 3, 2 << 3, 1 << 8
SHIFT_BEFORE, SHIFT_AFTER, SHIFT_LAST = 1 << 1, 1 << 5, 1 << 9
MRF_REPETITION = RELAX | ROTATE | RECORD | SHIFT_LAST
CPMG_REFOCUS = RELAX | SHIFT_BEFORE | ROTATE | SHIFT_AFTER
CPMG_RECORD = RELAX | RECORD


def _codes(events):
    from torchsim_gb300.batching import compile_ops

    return compile_ops(events)["code"].astype(np.int64)


def test_mrf_repetitions_take_the_straight_line_shape():
    from torchsim_gb300.sequence import mrf_events

    codes = _codes(mrf_events(mrf_schedule(), 10.0))
    assert codes.size == 881
    assert codes[0] == INVERT
    # The first pulse follows the inversion with no interval (TI = 0).
    assert codes[1] == MRF_REPETITION & ~RELAX
    assert np.all(codes[2:] == MRF_REPETITION)


def test_mrf_with_varying_tr_keeps_the_shape():
    from torchsim_gb300.sequence import mrf_events

    rng = np.random.default_rng(0)
    codes = _codes(mrf_events(rng.uniform(5, 70, 600).astype(np.float32),
                              rng.uniform(8, 15, 600).astype(np.float32), TI_ms=20.0))
    assert codes[0] == INVERT
    assert np.all(codes[1:] == MRF_REPETITION)


def test_cpmg_echoes_take_the_refocusing_and_recording_shapes():
    from torchsim_gb300.sequence import fse_events

    etl = 16
    codes = _codes(fse_events(np.full(etl, 150.0, np.float32), 10.0, phases_deg=90.0))
    assert codes.size == 1 + 2 * etl
    assert codes[0] == ROTATE  # the excitation
    assert np.all(codes[1::2] == CPMG_REFOCUS)
    assert np.all(codes[2::2] == CPMG_RECORD)
