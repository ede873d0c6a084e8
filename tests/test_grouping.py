"""Group matching on the host (no GPU): the reference's
estimators/_grouped.py contract, checked the way its tests/estimators/
test_grouped.py checks it on a synthetic two-parameter family of decays, and
pinned to the reference's own outputs on a committed fixture."""

from __future__ import annotations

import numpy as np
import pytest
import torch

from torchsim_gb300.matching import Grouping, correlate


@pytest.fixture(scope="module")
def family():
    """Inversion-recovery-like decays over a grid of two rates: neighbouring
    atoms are nearly parallel, as a simulated dictionary's are."""
    t = torch.linspace(0.01, 3.0, 120, dtype=torch.float64)
    r1 = torch.linspace(0.3, 5.0, 40, dtype=torch.float64)
    r2 = torch.linspace(1.0, 30.0, 25, dtype=torch.float64)
    g1, g2 = torch.meshgrid(r1, r2, indexing="ij")
    atoms = (1 - 2 * torch.exp(-t * g1.reshape(-1, 1))) * torch.exp(-t * g2.reshape(-1, 1) / 10)
    return atoms.to(torch.complex64) * (1 + 0.5j)


def test_every_atom_lands_in_exactly_one_group(family):
    grouping = Grouping.fit(family, 24)
    assigned = torch.cat(grouping.members).sort().values
    assert torch.equal(assigned, torch.arange(family.shape[0]))
    assert grouping.count == 24 and sum(grouping.sizes) == family.shape[0]


def test_groups_hold_a_full_share_but_the_last(family):
    grouping = Grouping.fit(family, 24)
    share = -(-family.shape[0] // 24)
    assert set(grouping.sizes[:-1]) == {share}
    assert 0 < grouping.sizes[-1] <= share


def test_a_group_keeps_its_atoms_normalized_in_their_own_basis(family):
    grouping = Grouping.fit(family, 24)
    members = family[grouping.members[0]]
    want = members / torch.linalg.vector_norm(members, dim=-1, keepdim=True)
    torch.testing.assert_close(grouping.atoms[0], want)
    assert grouping.atoms[0].shape[-1] == family.shape[-1]


def test_the_first_group_is_seeded_by_the_first_atom_and_holds_its_nearest(family):
    grouping = Grouping.fit(family, 24)
    first = grouping.members[0]
    assert 0 in first.tolist()
    unit = family / torch.linalg.vector_norm(family, dim=-1, keepdim=True)
    alike = (unit @ unit[0].conj()).abs()
    outside = torch.ones(family.shape[0], dtype=torch.bool)
    outside[first] = False
    assert float(alike[first].min()) >= float(alike[outside].max())


def test_representatives_are_unit_group_means(family):
    grouping = Grouping.fit(family, 8)
    for g in range(grouping.count):
        mean = grouping.atoms[g].mean(0)
        torch.testing.assert_close(grouping.representative[g], mean / torch.linalg.vector_norm(mean))


def test_the_condition_number_climbs_with_the_group_count(family):
    few = Grouping.fit(family, 4).condition
    many = Grouping.fit(family, 64).condition
    assert few > 1.0 and many > few


def test_as_many_groups_as_atoms_gives_one_each(family):
    grouping = Grouping.fit(family, family.shape[0])
    assert grouping.count == family.shape[0] and set(grouping.sizes) == {1}


@pytest.mark.parametrize("count", [0, 10**6])
def test_a_group_count_out_of_range_is_refused(family, count):
    with pytest.raises(ValueError):
        Grouping.fit(family, count)


def test_survivors_keep_the_best_group_and_widen_with_the_threshold(family):
    grouping = Grouping.fit(family, 24)
    gen = torch.Generator().manual_seed(7)
    picked = family[::37]
    noise = torch.randn(picked.shape, generator=gen, dtype=torch.complex64)
    signals = picked + 0.01 * float(family.abs().max()) * noise
    signals = signals / torch.linalg.vector_norm(signals, dim=-1, keepdim=True)
    tight = grouping.survivors(signals, 0.0)
    loose = grouping.survivors(signals, 0.2)
    assert bool(tight.any(-1).all())
    assert bool((loose | ~tight).all())  # loose keeps every group tight keeps
    assert float(loose.sum(-1).float().mean()) > float(tight.sum(-1).float().mean())
    best = correlate(signals, grouping.representative).argmax(-1)
    assert bool(tight[torch.arange(signals.shape[0]), best].all())


def test_correlate_is_blind_to_complex_scale(family):
    unit = family / torch.linalg.vector_norm(family, dim=-1, keepdim=True)
    turned = unit[:5] * (0.3 - 0.7j) / abs(0.3 - 0.7j)
    torch.testing.assert_close(correlate(turned, unit), correlate(unit[:5], unit))
    real = unit.real / torch.linalg.vector_norm(unit.real, dim=-1, keepdim=True)
    both = correlate(turned, real)
    assert both.shape == (5, family.shape[0]) and bool((both >= 0).all())


def test_grouping_matches_the_reference(golden):
    """The reference's own Grouping.fit, survivors and match_in_groups on the
    same family (tests/golden/grouping.npz, made by tests/golden/
    make_golden.py from estimators/_grouped.py): the same groups, the same
    representatives, the same surviving groups at three thresholds and the
    same top-3 grouped match."""
    from torchsim_gb300.matching import _search_groups

    d = golden("grouping")
    atoms = torch.from_numpy(d["atoms"])
    grouping = Grouping.fit(atoms, 24)
    assert list(grouping.sizes) == d["sizes"].tolist()
    offsets = np.concatenate([[0], np.cumsum(d["sizes"])])
    for g, members in enumerate(grouping.members):
        want = d["members"][offsets[g]:offsets[g + 1]]
        assert sorted(members.tolist()) == sorted(want.tolist()), g
    torch.testing.assert_close(grouping.representative, torch.from_numpy(d["representative"]),
                               rtol=1e-5, atol=1e-6)
    assert grouping.condition == pytest.approx(float(d["condition"]), rel=1e-4)
    signals = torch.from_numpy(d["signals"])
    unit = signals / torch.linalg.vector_norm(signals, dim=-1, keepdim=True)
    for prune in (0.0, 5e-3, 0.2):
        got = grouping.survivors(unit, prune).numpy()
        assert np.array_equal(got, d[f"survivors_{prune:g}"]), prune
    indices, scores = _search_groups(unit, grouping, 3, 5e-3)
    assert np.array_equal(indices.numpy(), d["match_indices"])
    np.testing.assert_allclose(scores.numpy(), d["match_scores"], rtol=1e-5, atol=1e-6)
