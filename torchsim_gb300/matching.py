"""Dictionary matching: the best atoms of a simulated dictionary per voxel.

The interface is the reference's ``DictionaryMatcher`` / ``MatchResult``
(``estimators/_dictionary.py:18-420``): atoms and signals are normalized, a
voxel's score against an atom is ``|<s, d>|`` (``_grouped.py:212-240``), and a
match returns the top-k atoms with their scores, the complex least-squares
scale (proton density and receive phase), its size and the atoms' parameter
values.

The search is one tensor-core kernel per chunk of voxels
(``tsg_match_screen``): fp16 products accumulated in FP32 in tensor memory,
with the selection of each voxel's best 32 atoms fused into the epilogue, so
the voxel x atom score matrix never exists. Each atom enters the screen as two
fp16 rows (its value and the rounding remainder), so the screen's scores carry
the atoms to ~22 bits and only the query's rounding, which shifts near-parallel
atoms alike, is left. The candidates are then rescored exactly in FP32 against
the complex signals (``tsg_match_rescore``) and the top k kept, so the screen
only narrows which atoms are compared exactly.

Group matching (``groups``) is the reference's option for dictionaries too
large to search exhaustively (``estimators/_grouped.py``; Cauley, Setsompop,
Ma et al., "Fast group matching for MR fingerprinting reconstruction", MRM
74(2), 2015): the dictionary is clustered into groups of nearly parallel
atoms, a voxel is scored against each group's representative first, and only
the groups within ``prune`` of its best representative score are searched.
It is approximate (a pruned group may hold the best atom) and kept for the
reference's semantics; on this GPU the exhaustive tensor-core search is exact
and faster.
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass

import torch

from . import _native, engine

__all__ = ["DictionaryMatcher", "Grouping", "MatchResult", "correlate"]


@dataclass(frozen=True)
class MatchResult:
    """Best atoms per voxel (``(..., k)``): ``parameters`` ``(..., k, n)`` (or
    None without parameter values), ``indices``, ``scores`` (the normalized
    ``|<s, d>|``), ``scales`` (complex least-squares scale) and ``densities``
    (``|scale|``)."""

    parameters: torch.Tensor | None
    indices: torch.Tensor
    scores: torch.Tensor
    scales: torch.Tensor
    densities: torch.Tensor


def _normalized(x: torch.Tensor) -> tuple[torch.Tensor, torch.Tensor]:
    norm = torch.linalg.vector_norm(x, dim=-1).clamp_min(torch.finfo(torch.float32).eps)
    return x / norm[:, None], norm


def correlate(signals: torch.Tensor, atoms: torch.Tensor) -> torch.Tensor:
    """``|<s, d>|`` of every (normalized) signal against every (normalized)
    atom, ``(voxels, atoms)`` real: blind to the complex scale that proton
    density and receive phase put on a signal (``_grouped.py:212-243``). A
    complex signal against real atoms scores both of its parts."""
    if torch.is_complex(signals) and not torch.is_complex(atoms):
        return torch.hypot(signals.real @ atoms.mT, signals.imag @ atoms.mT)
    return (signals @ atoms.mH).abs()


@dataclass(frozen=True)
class Grouping:
    """A dictionary split into groups of nearly parallel atoms
    (``_grouped.py:34-161``): ``members`` the atom indices of each group,
    ``representative`` ``(groups, contrasts)`` each group's unit mean signal,
    ``atoms`` each group's unit atoms in the dictionary's own basis."""

    members: tuple[torch.Tensor, ...]
    representative: torch.Tensor
    atoms: tuple[torch.Tensor, ...]

    @property
    def count(self) -> int:
        return len(self.members)

    @property
    def sizes(self) -> tuple[int, ...]:
        return tuple(int(m.numel()) for m in self.members)

    @property
    def condition(self) -> float:
        """Condition number of the representatives: it climbs once groups
        start to look alike, which is when there are too many to prune with."""
        s = torch.linalg.svdvals(self.representative.to(torch.complex64))
        return float(s[0] / s[-1].clamp_min(torch.finfo(torch.float32).tiny))

    @classmethod
    def fit(cls, dictionary: torch.Tensor, count: int) -> Grouping:
        """Greedy clustering into ``count`` groups (``_grouped.py:76-131``):
        the first atom not yet in a group seeds one and takes the
        ceil(atoms / count) unassigned atoms most correlated with it
        (itself among them); repeated until every atom has a group, so all
        groups but the last hold a full share."""
        total = int(dictionary.shape[0])
        if not 1 <= count <= total:
            raise ValueError(f"count must be between one and the {total} atoms, got {count}")
        unit = dictionary
        if not (torch.is_complex(unit) or torch.is_floating_point(unit)):
            unit = unit.to(torch.float32)
        unit, _ = _normalized(unit)
        share = -(-total // count)
        free = torch.ones(total, dtype=torch.bool, device=unit.device)
        floor = torch.full((total,), -1.0, dtype=unit.real.dtype, device=unit.device)
        members = []
        left = total
        while left:
            seed = int(torch.argmax(free.to(torch.int8)))  # the first free atom
            alike = torch.where(free, (unit @ unit[seed].conj()).abs(), floor)
            take = min(share, left)
            chosen = torch.topk(alike, take).indices
            members.append(chosen)
            free[chosen] = False
            left -= take
        representative = torch.cat([_normalized(unit[m].mean(0, keepdim=True))[0] for m in members])
        return cls(members=tuple(members), representative=representative,
                   atoms=tuple(unit[m] for m in members))

    def survivors(self, signals: torch.Tensor, prune: float) -> torch.Tensor:
        """``(voxels, groups)`` bool: the groups whose representative scores
        within ``prune`` (a fraction) of a voxel's best representative score
        (``_grouped.py:133-151``). ``signals`` are normalized."""
        scores = correlate(signals, self.representative)
        return scores >= scores.amax(-1, keepdim=True) * (1.0 - prune)

    def to(self, device: torch.device) -> Grouping:
        if self.representative.device == torch.device(device):
            return self
        return Grouping(members=tuple(m.to(device) for m in self.members),
                        representative=self.representative.to(device),
                        atoms=tuple(x.to(device) for x in self.atoms))


def _search_groups(signals: torch.Tensor, grouping: Grouping, top_k: int,
                   prune: float) -> tuple[torch.Tensor, torch.Tensor]:
    """Top-k atoms and scores of normalized ``signals`` within each voxel's
    surviving groups (``_grouped.py:164-209``): every group that some voxel
    kept is scored against those voxels only, and its best k merge into the
    voxels' running top k."""
    V = signals.shape[0]
    scores = torch.full((V, top_k), -1.0, dtype=signals.real.dtype, device=signals.device)
    indices = torch.zeros((V, top_k), dtype=torch.int64, device=signals.device)
    keep = grouping.survivors(signals, prune)
    for g in torch.nonzero(keep.any(0)).flatten().tolist():
        rows = torch.nonzero(keep[:, g]).flatten()
        local = correlate(signals[rows], grouping.atoms[g])
        found, where = torch.topk(local, min(top_k, local.shape[1]), dim=-1)
        pool_scores = torch.cat((scores[rows], found), dim=-1)
        pool_indices = torch.cat((indices[rows], grouping.members[g][where]), dim=-1)
        best, pick = torch.topk(pool_scores, top_k, dim=-1)
        scores[rows] = best
        indices[rows] = torch.gather(pool_indices, -1, pick)
    return indices, scores


def _pad8(x: torch.Tensor) -> torch.Tensor:
    extra = (-x.shape[-1]) % 8
    return torch.nn.functional.pad(x, (0, extra)) if extra else x


class DictionaryMatcher:
    """Match signals against ``dictionary`` ``(atoms, contrasts)`` by normalized
    complex inner products; ``parameters`` ``(atoms, n)`` are returned for the
    matched atoms. ``top_k`` (1..8) candidates per voxel; voxels are matched
    ``query_chunk_size`` at a time. ``groups`` clusters the dictionary into
    that many groups (at most one per atom) and searches only the groups
    within ``prune`` of a voxel's best group (:class:`Grouping`; read
    :attr:`grouping` after fitting)."""

    def __init__(self, acquisition=None, *, dictionary: torch.Tensor | None = None,
                 parameters: torch.Tensor | None = None, query_chunk_size: int = 65536,
                 dictionary_chunk_size: int = 16384, top_k: int = 1, groups: int | None = None,
                 prune: float = 5e-3, device: torch.device | str | None = None) -> None:
        if acquisition is not None:
            raise NotImplementedError("simulate the dictionary first and pass dictionary=")
        if groups is not None and groups < 1:
            raise ValueError(f"groups must be positive, got {groups}")
        if query_chunk_size < 1 or dictionary_chunk_size < 1:
            raise ValueError("chunk sizes must be positive")
        if not 1 <= top_k <= 8:
            raise ValueError("top_k must be between 1 and 8")
        if not 0.0 <= prune < 1.0:
            raise ValueError(f"prune must be in [0, 1), got {prune}")
        self.query_chunk_size = int(query_chunk_size)
        self.dictionary_chunk_size = int(dictionary_chunk_size)
        self.top_k = int(top_k)
        self.groups = None if groups is None else int(groups)
        self.prune = float(prune)
        self.grouping: Grouping | None = None
        self.device = engine.require_cuda(torch.device(device) if device is not None else None)
        self.dictionary = None
        if dictionary is not None:
            self.fit(dictionary, parameters)

    @property
    def fitted(self) -> bool:
        return self.dictionary is not None

    def fit(self, dictionary: torch.Tensor, parameters: torch.Tensor | None = None):
        """Adopt ``dictionary`` (and the parameter values of its atoms)."""
        d = torch.as_tensor(dictionary)
        if d.ndim != 2 or d.shape[0] < 1:
            raise ValueError("dictionary must have shape (atoms, contrasts)")
        if self.top_k > d.shape[0]:
            raise ValueError("top_k must be between one and the atom count")
        d = d.to(self.device, torch.complex64)
        self.dictionary = d
        self.normalized, norm = _normalized(d)
        self.power = norm.square()
        re, im = self.normalized.real, self.normalized.imag
        # A real dictionary (or one on the imaginary axis, as the MRF signal
        # 1j*s is) scores like its real profile: |<s, e^{i c} d>| = |<s, d>|.
        if not bool(im.ne(0).any()):
            self._screen_atoms, self._complex_atoms = re, False
        elif not bool(re.ne(0).any()):
            self._screen_atoms, self._complex_atoms = im, False
        else:
            self._screen_atoms, self._complex_atoms = torch.cat((re, im), dim=1), True
        # Each screen atom is a pair of fp16 rows, hi and lo = (atom - hi),
        # side by side along the contraction: the query meets both, so its
        # product is <q, atom> with the atom carried to ~22 bits. What rounding
        # is left is the query's own, and that error is common to every atom
        # of a voxel: <q - s, d1 - d2> is tiny for two nearly parallel atoms,
        # so the screen ranks neighbours of a dense dictionary the way the
        # exact scores do. Values are scaled by sqrt(contrasts) first so that
        # the lo parts stay clear of fp16's subnormal range.
        self._screen_scale = float(self._screen_atoms.shape[1]) ** 0.5
        scaled = self._screen_atoms * self._screen_scale
        hi = scaled.to(torch.float16)
        lo = (scaled - hi.float()).to(torch.float16)
        screen = torch.cat((_pad8(hi), _pad8(lo)), dim=1)
        # The kernel reads atom i from row pos(i) (bit 1 of i moved to bit 5,
        # bits 2-5 down by one, within blocks of 64) of a matrix padded to a
        # multiple of 64 rows, so neighbouring atoms fall in different
        # candidate lists.
        A = screen.shape[0]
        rows = int(_native.library().tsg_match_screen_rows(A))
        i = torch.arange(A, device=self.device)
        pos = (i & 1) | (((i >> 1) & 1) << 5) | (((i >> 2) & 15) << 1) | (i & ~63)
        stored = torch.zeros((rows, screen.shape[1]), dtype=torch.float16, device=self.device)
        stored[pos] = screen
        self._screen_atoms = stored
        self.grouping = (None if self.groups is None
                         else Grouping.fit(d, min(self.groups, d.shape[0])))
        if parameters is None:
            self.parameter_values = None
        else:
            p = torch.as_tensor(parameters, dtype=torch.float32, device=self.device)
            p = p[:, None] if p.ndim == 1 else p
            if p.ndim != 2 or p.shape[0] != d.shape[0]:
                raise ValueError("parameters must have shape (atoms, parameters)")
            self.parameter_values = p
        return self

    def _queries(self, s: torch.Tensor) -> torch.Tensor:
        """Two fp16 rows per voxel whose products with the screen atoms are
        Re and Im of <s, d>."""
        if self._complex_atoms:
            a = torch.cat((s.real, s.imag), dim=1)
            b = torch.cat((s.imag, -s.real), dim=1)
        else:
            a, b = s.real, s.imag
        rows = torch.stack((a, b), dim=1).reshape(2 * s.shape[0], a.shape[1])
        rows = _pad8(rows * self._screen_scale).to(torch.float16)
        return torch.cat((rows, rows), dim=1).contiguous()

    @torch.no_grad()
    def match(self, signals: torch.Tensor) -> MatchResult:
        """Top-k atoms, scores, scales, densities and parameters per voxel."""
        if not self.fitted:
            raise RuntimeError("the matcher has no dictionary to match against")
        signals = torch.as_tensor(signals)
        if signals.shape[-1] != self.dictionary.shape[-1]:
            raise ValueError("signal and dictionary contrast counts differ")
        sample_shape = signals.shape[:-1]
        flat = signals.reshape(-1, signals.shape[-1]).to(self.device, torch.complex64)
        lib = _native.library()
        stream = torch.cuda.current_stream(self.device).cuda_stream
        A, P = self.dictionary.shape
        screen_k = self._screen_atoms.shape[1]  # rows: the padded, permuted atoms
        m = lib.tsg_match_candidates()
        error = torch.zeros(1, dtype=torch.int32, device=self.device)
        scores, indices = [], []
        for chunk in flat.split(self.query_chunk_size):
            V = chunk.shape[0]
            s_hat, _ = _normalized(chunk)
            if self.grouping is not None:
                ix, sc = _search_groups(s_hat, self.grouping, self.top_k, self.prune)
                scores.append(sc)
                indices.append(ix)
                continue
            queries = self._queries(s_hat)
            cand_s = torch.empty((V, m), dtype=torch.float32, device=self.device)
            cand_i = torch.empty((V, m), dtype=torch.int32, device=self.device)
            _native.check(lib.tsg_match_screen(
                queries.data_ptr(), 2 * V, self._screen_atoms.data_ptr(), A, screen_k,
                cand_s.data_ptr(), cand_i.data_ptr(), error.data_ptr(), stream))
            sc = torch.empty((V, self.top_k), dtype=torch.float32, device=self.device)
            ix = torch.empty((V, self.top_k), dtype=torch.int64, device=self.device)
            s_hat = s_hat.contiguous()
            _native.check(lib.tsg_match_rescore(
                s_hat.data_ptr(), V, self.normalized.data_ptr(), A, P, cand_i.data_ptr(),
                self.top_k, sc.data_ptr(), ix.data_ptr(), stream))
            scores.append(sc)
            indices.append(ix)
        if int(error.item()) != 0:
            raise _native.NativeError(_native.TSG_ERR_CUDA,
                                      f"matching kernel stopped waiting (stage {int(error.item())})")
        scores = torch.cat(scores) if scores else torch.empty((0, self.top_k), device=self.device)
        indices = (torch.cat(indices) if indices
                   else torch.empty((0, self.top_k), dtype=torch.int64, device=self.device))
        signal_norm = torch.linalg.vector_norm(flat, dim=-1).clamp_min(torch.finfo(torch.float32).eps)
        densities = signal_norm[:, None] * scores / self.power[indices].sqrt()
        atoms = self.dictionary[indices]
        scales = torch.sum(atoms.conj() * flat[:, None, :], dim=-1) / self.power[indices]
        shape = (*sample_shape, self.top_k)
        params = None
        if self.parameter_values is not None:
            params = self.parameter_values[indices].reshape(*shape, self.parameter_values.shape[-1])
        return MatchResult(parameters=params, indices=indices.reshape(shape),
                           scores=scores.reshape(shape), scales=scales.reshape(shape),
                           densities=densities.reshape(shape))

    def __call__(self, signals: torch.Tensor) -> torch.Tensor:
        """Best parameter values (indices without parameters), per voxel."""
        result = self.match(signals)
        if result.parameters is None:
            return result.indices[..., 0]
        return result.parameters[..., 0, :]
