"""Dictionary matching on the tensor cores against an exhaustive FP64 search
(the reference's DictionaryMatcher semantics, estimators/_dictionary.py:
329-420: normalized |<s, d>|, top-k, least-squares scale and density)."""

from __future__ import annotations

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def exhaustive(signals: np.ndarray, atoms: np.ndarray, k: int):
    s = signals.astype(np.complex128)
    d = atoms.astype(np.complex128)
    sn = s / np.maximum(np.linalg.norm(s, axis=1, keepdims=True), 1e-30)
    dn = d / np.maximum(np.linalg.norm(d, axis=1, keepdims=True), 1e-30)
    scores = np.abs(sn @ dn.conj().T)
    order = np.argsort(-scores, axis=1, kind="stable")[:, :k]
    return scores, order


def make_case(rng, V, A, P, kind):
    if kind == "real":
        atoms = rng.standard_normal((A, P)).astype(np.float32).astype(np.complex64)
    elif kind == "imaginary":
        atoms = (1j * rng.standard_normal((A, P))).astype(np.complex64)
    else:
        atoms = (rng.standard_normal((A, P)) + 1j * rng.standard_normal((A, P))).astype(np.complex64)
    truth = rng.integers(0, A, V)
    scale = (rng.uniform(0.5, 2.0, V) * np.exp(1j * rng.uniform(-np.pi, np.pi, V)))
    noise = 0.05 * (rng.standard_normal((V, P)) + 1j * rng.standard_normal((V, P)))
    signals = (atoms[truth] * scale[:, None] + noise * np.abs(atoms).mean()).astype(np.complex64)
    return signals, atoms, truth


@pytest.mark.parametrize("kind", ["real", "imaginary", "complex"])
@pytest.mark.parametrize("V,A,P", [(300, 1000, 100), (64, 37, 880), (1, 5, 8)])
def test_match_equals_exhaustive_search(cuda, kind, V, A, P):
    from torchsim_gb300 import DictionaryMatcher

    rng = np.random.default_rng(V + A + P)
    signals, atoms, truth = make_case(rng, V, A, P, kind)
    k = min(3, A)
    params = rng.uniform(0, 1, (A, 2)).astype(np.float32)
    matcher = DictionaryMatcher(dictionary=torch.from_numpy(atoms), parameters=torch.from_numpy(params),
                                top_k=k, query_chunk_size=128)
    res = matcher.match(torch.from_numpy(signals).to(cuda))
    scores, order = exhaustive(signals, atoms, k)
    idx = res.indices.cpu().numpy()
    got = res.scores.cpu().numpy()
    best = scores[np.arange(V), order[:, 0]]
    # The chosen atoms score what the FP64 search says they score ...
    assert np.abs(got - np.take_along_axis(scores, idx, 1)).max() <= 2e-6
    # ... and the first is the best, up to FP32 ties.
    assert np.all(scores[np.arange(V), idx[:, 0]] >= best - 2e-6)
    assert np.mean(idx[:, 0] == order[:, 0]) >= 0.99
    if A > 1:
        assert np.all(np.diff(got, axis=1) <= 1e-7)  # best first
    # Least-squares scale and density of the first candidate.
    d = atoms[idx[:, 0]].astype(np.complex128)
    scale = np.sum(d.conj() * signals, axis=1) / np.sum(np.abs(d) ** 2, axis=1)
    assert np.abs(res.scales[:, 0].cpu().numpy() - scale).max() <= 1e-4 * np.abs(scale).max()
    assert np.abs(res.densities[:, 0].cpu().numpy() - np.abs(scale)).max() <= 1e-4 * np.abs(scale).max()
    np.testing.assert_array_equal(res.parameters.cpu().numpy(), params[idx])


def test_match_recovers_mrf_dictionary_atoms(cuda):
    """A dictionary from the MRF simulator (on the imaginary axis) and noisy,
    scaled, phase-turned signals of its own atoms."""
    import torchsim_gb300 as ts

    rng = np.random.default_rng(3)
    flip = np.concatenate([np.linspace(5, 60, 100), np.linspace(60, 2, 100)]).astype(np.float32)
    t1 = np.geomspace(100, 4000, 40)
    t2 = np.geomspace(5, 500, 30)
    g1, g2 = np.meshgrid(t1, t2, indexing="ij")
    keep = g2 < g1
    T1 = torch.from_numpy(g1[keep].astype(np.float32)).to(cuda)
    T2 = torch.from_numpy(g2[keep].astype(np.float32)).to(cuda)
    dictionary = ts.mrf_sim(torch.from_numpy(flip), 10.0, T1, T2, states=10)
    matcher = ts.DictionaryMatcher(dictionary=dictionary, parameters=torch.stack((T1, T2), 1))
    truth = rng.integers(0, dictionary.shape[0], 500)
    phase = torch.from_numpy(np.exp(1j * rng.uniform(-3, 3, 500)).astype(np.complex64)).to(cuda)
    noise = torch.from_numpy((rng.standard_normal((500, 200)) + 1j * rng.standard_normal((500, 200)))
                             .astype(np.complex64)).to(cuda) * 1e-3
    measured = dictionary[torch.from_numpy(truth).to(cuda)] * (0.7 * phase[:, None]) + noise
    maps = matcher(measured)
    got = maps.cpu().numpy()
    want = np.stack((g1[keep], g2[keep]), 1)[truth]
    assert np.mean(np.all(np.isclose(got, want, rtol=1e-5), axis=1)) >= 0.99
    res = matcher.match(measured)
    np.testing.assert_allclose(res.densities[:, 0].cpu().numpy(), 0.7, rtol=2e-2)


def test_match_argument_errors(cuda):
    from torchsim_gb300 import DictionaryMatcher

    atoms = torch.ones((4, 16), dtype=torch.complex64)
    with pytest.raises(ValueError):
        DictionaryMatcher(dictionary=atoms, top_k=9)
    with pytest.raises(ValueError):
        DictionaryMatcher(dictionary=atoms, groups=0)
    with pytest.raises(ValueError):
        DictionaryMatcher(dictionary=atoms, prune=1.0)
    m = DictionaryMatcher(dictionary=atoms)
    with pytest.raises(ValueError):
        m.match(torch.ones((3, 15), dtype=torch.complex64))


# ---- group matching (the reference's tests/estimators/test_grouped.py) -------


@pytest.fixture(scope="module")
def fingerprints(cuda):
    """An MRF dictionary over a 60 x 30 T1/T2 grid (200 flips U(10, 60) deg,
    TR 10 ms, TI 20 ms) and a noisy off-grid volume of every 37th atom."""
    import torchsim_gb300 as ts

    gen = torch.Generator().manual_seed(0)
    flip = 10.0 + 50.0 * torch.rand(200, generator=gen)
    grid = torch.cartesian_prod(torch.linspace(200.0, 3000.0, 60), torch.linspace(20.0, 300.0, 30))
    atoms = ts.mrf_sim(flip, 10.0, grid[:, 0].to(cuda), grid[:, 1].to(cuda), TI=20.0, states=10)
    noise_gen = torch.Generator().manual_seed(7)
    picked = atoms[::37]
    noise = torch.randn(picked.shape, generator=noise_gen, dtype=torch.complex64).to(cuda)
    measured = picked + 0.01 * float(atoms.abs().max()) * noise
    return atoms, grid.to(cuda), measured


def test_grouped_matching_finds_what_direct_matching_finds(fingerprints):
    """Where the pruned search differs from the exhaustive one it is by a grid
    step: at least 80% agree and the mean relative error stays under 1%."""
    from torchsim_gb300 import DictionaryMatcher

    atoms, grid, measured = fingerprints
    direct = DictionaryMatcher(dictionary=atoms, parameters=grid)(measured)
    grouped = DictionaryMatcher(dictionary=atoms, parameters=grid, groups=24)(measured)
    assert float((direct == grouped).all(-1).float().mean()) > 0.8
    for column in range(grid.shape[-1]):
        error = ((grouped[:, column] - direct[:, column]) / direct[:, column]).abs()
        assert float(error.mean()) < 0.01


def test_grouped_matching_rules_out_most_of_the_dictionary(fingerprints):
    from torchsim_gb300 import DictionaryMatcher

    atoms, grid, measured = fingerprints
    matcher = DictionaryMatcher(dictionary=atoms, parameters=grid, groups=24)
    unit = measured / torch.linalg.vector_norm(measured, dim=-1, keepdim=True)
    kept = matcher.grouping.survivors(unit, matcher.prune)
    assert float(kept.sum(-1).float().mean()) < 0.25 * matcher.grouping.count
    assert float(matcher.grouping.survivors(unit, 0.2).sum(-1).float().mean()) > float(
        matcher.grouping.survivors(unit, 0.0).sum(-1).float().mean())


def test_grouped_scores_are_the_exact_scores_of_the_atoms_found(fingerprints):
    """Whatever atom the pruned search returns, its score is that atom's
    exact normalized correlation, and the top k come ranked."""
    from torchsim_gb300 import DictionaryMatcher
    from torchsim_gb300.matching import correlate

    atoms, grid, measured = fingerprints
    matcher = DictionaryMatcher(dictionary=atoms, parameters=grid, groups=24, top_k=3)
    found = matcher.match(measured)
    assert found.indices.shape == (measured.shape[0], 3)
    assert bool((torch.diff(found.scores, dim=-1) <= 1e-5).all())
    assert bool((found.indices < atoms.shape[0]).all())
    unit_s = measured / torch.linalg.vector_norm(measured, dim=-1, keepdim=True)
    unit_a = atoms / torch.linalg.vector_norm(atoms, dim=-1, keepdim=True)
    exact = torch.gather(correlate(unit_s, unit_a), 1, found.indices)
    torch.testing.assert_close(found.scores, exact, rtol=1e-5, atol=1e-6)
    torch.testing.assert_close(found.parameters, grid[found.indices])


def test_more_groups_than_atoms_gives_one_each(fingerprints):
    from torchsim_gb300 import DictionaryMatcher

    atoms, grid, measured = fingerprints
    few = atoms[:10]
    matcher = DictionaryMatcher(dictionary=few, parameters=grid[:10], groups=50)
    assert matcher.grouping.count == 10
    exhaustive = DictionaryMatcher(dictionary=few, parameters=grid[:10])
    # One atom per group and nothing pruned: the exhaustive answer.
    got = DictionaryMatcher(dictionary=few, parameters=grid[:10], groups=50, prune=0.999)
    assert torch.equal(got.match(measured).indices, exhaustive.match(measured).indices)


def fp64_best_two(signals: torch.Tensor, atoms: torch.Tensor, chunk: int = 16384):
    """FP64 exhaustive search on the device: each signal's best and second
    best normalized |<s, d>| over every atom, and the best atom. ``atoms``
    are real profiles (a dictionary on one axis of the complex plane scores
    as its profile: |<s, 1j d>| = |<s, d>|)."""
    s = signals.to(torch.complex128)
    s = s / torch.linalg.vector_norm(s, dim=-1, keepdim=True)
    sr, si = s.real.contiguous(), s.imag.contiguous()
    V = s.shape[0]
    top = torch.full((V, 2), -1.0, dtype=torch.float64, device=s.device)
    arg = torch.zeros((V, 2), dtype=torch.int64, device=s.device)
    for start in range(0, atoms.shape[0], chunk):
        d = atoms[start:start + chunk].to(torch.float64)
        d = d / torch.linalg.vector_norm(d, dim=-1, keepdim=True)
        sc = torch.hypot(sr @ d.T, si @ d.T)
        v, i = torch.topk(sc, 2, dim=1)
        pool_v = torch.cat((top, v), dim=1)
        pool_i = torch.cat((arg, i + start), dim=1)
        top, pick = torch.topk(pool_v, 2, dim=1)
        arg = torch.gather(pool_i, 1, pick)
    return top, arg


def test_match_on_the_dictionary_workload_equals_fp64_argmax(cuda):
    """The benchmark's matching workload: 4,096 voxels of SNR-50 signal
    (random true atom, random phase) against the full 262,144-atom MRF
    dictionary (880 pulses, 20 states), whose nearest neighbours are nearly
    parallel. The top-1 atom equals the FP64 exhaustive argmax wherever the
    FP64 best and second best are further apart than FP32 rounding of the
    exact rescoring can blur (2e-6 of a unit score), and the chosen atom never
    scores more than 1e-6 below the FP64 best."""
    from torchsim_gb300 import DictionaryMatcher, engine
    from torchsim_gb300.sequence import mrf_events, program_for
    from tests.helpers import mrf_schedule

    t1 = np.geomspace(100, 4000, 128, dtype=np.float32)
    t2 = np.geomspace(5, 500, 64, dtype=np.float32)
    b1 = np.linspace(0.6, 1.4, 32, dtype=np.float32)
    T1, T2, B1 = (torch.from_numpy(np.ascontiguousarray(a.reshape(-1)))
                  for a in np.meshgrid(t1, t2, b1, indexing="ij"))
    A = T1.numel()
    prog = program_for(mrf_events(mrf_schedule(), 10.0), cuda)
    dictionary = engine.forward(prog, engine.tissue_maps(cuda, A, T1, T2, None, B1, None), 20)
    matcher = DictionaryMatcher(dictionary=dictionary, query_chunk_size=4096)
    rng = np.random.default_rng(11)
    V = 4096
    truth = torch.from_numpy(rng.integers(0, A, V)).to(cuda)
    phase = torch.from_numpy(np.exp(1j * rng.uniform(-np.pi, np.pi, V)).astype(np.complex64)).to(cuda)
    sig = dictionary[truth] * phase[:, None]
    g = torch.Generator(device=cuda).manual_seed(11)
    sigma = float(sig.abs().mean()) / 50.0
    noise = torch.complex(torch.randn(sig.shape, device=cuda, generator=g),
                          torch.randn(sig.shape, device=cuda, generator=g)) * (sigma / 2 ** 0.5)
    res = matcher.match(sig + noise)
    # The dictionary lies on one axis of the complex plane (the public MRF
    # signal is real): its profile on that axis.
    profile = dictionary.imag if bool(dictionary.imag.ne(0).any()) else dictionary.real
    assert not bool((dictionary.imag.ne(0) & dictionary.real.ne(0)).any())
    top, arg = fp64_best_two(sig + noise, profile)
    chosen = res.indices[:, 0]
    separated = (top[:, 0] - top[:, 1]) > 2e-6
    assert bool(separated.float().mean() > 0.5)
    assert torch.equal(chosen[separated], arg[separated, 0])
    # The chosen atom's own FP64 score, against the best.
    s = (sig + noise).to(torch.complex128)
    s = s / torch.linalg.vector_norm(s, dim=-1, keepdim=True)
    d = profile[chosen].to(torch.float64)
    d = d / torch.linalg.vector_norm(d, dim=-1, keepdim=True)
    own = torch.hypot((s.real * d).sum(-1), (s.imag * d).sum(-1))
    assert float((top[:, 0] - own).max()) <= 1e-6
    assert float((chosen == arg[:, 0]).float().mean()) >= 0.999
