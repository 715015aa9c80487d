"""gdock_gb300: GB300-native population fitness evaluation and FCC clustering
for the gdock protein-protein docker.

The compute runs in ``libgdock_gb300.so`` (CUDA, sm_103a) behind the C ABI of
``include/gdock_gb300.h``; this package is the thin Python view of that ABI
used by the tests and the benchmark, with the reference's names:

* ``Complex.score_poses``  -> Population::eval_fitness (src/population.rs:48-61)
* ``Complex.score_models`` -> commands::score::score (src/commands/score.rs:32-79)
* ``vdw_energy`` / ``elec_energy`` / ``desolv_energy`` / ``air_energy`` /
  ``satisfaction_ratio`` -> src/fitness.rs
* ``Complex.pose_contacts`` -> clustering::calculate_contacts (src/clustering.rs:62-115)
* ``Complex.cluster`` / ``cluster_sets`` -> clustering::cluster_structures
  (src/clustering.rs:265-293)
* ``Evaluator`` -> evaluator::Evaluator (src/evaluator.rs:50-144);
  ``Evaluator.eval_metrics`` -> Population::eval_metrics (src/population.rs:63-71)
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import List, Optional, Sequence, Tuple

import numpy as np

from . import _lib
from ._lib import (DOCK_METRICS_DTYPE, HOF_ENTRY_DTYPE, GD_PREC_F32, GD_PREC_F64, Context, GdError, POSE_ENERGY_DTYPE, PackedAtoms,
                   ga_default_cfg, ga_draw, make_frames, pack_names, ptr)
from .pdb import Molecule, combine_molecules, position_ligand, read_pdb, read_pdb_text

__all__ = [
    "Context", "Complex", "GdError", "GD_PREC_F32", "GD_PREC_F64", "EnergyWeights", "ClusteringConfig",
    "ClusterResult", "vdw_energy", "elec_energy", "desolv_energy", "air_energy", "satisfaction_ratio",
    "cluster_sets", "make_frames", "Molecule", "read_pdb", "read_pdb_text", "position_ligand",
    "combine_molecules", "default_context", "ga_default_cfg", "ga_draw", "run_ga", "GaResult", "Server",
    "Evaluator", "Metrics",
]


@dataclass
class EnergyWeights:
    """src/constants.rs:28-56"""
    vdw: float = 0.4
    elec: float = 0.05
    desolv: float = 3.4
    air: float = 1.0


@dataclass
class ClusteringConfig:
    """src/clustering.rs:14-35"""
    contact_distance: float = 5.0
    fcc_cutoff: float = 0.60
    strictness: float = 0.75
    min_cluster_size: int = 4

    def c(self):
        return _lib.GdClusterCfg(self.contact_distance, self.fcc_cutoff, self.strictness, self.min_cluster_size)


@dataclass
class ClusterResult:
    """src/clustering.rs:38-46"""
    center_idx: int
    members: List[int]
    size: int


_default_ctx: Optional[Context] = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


def _prec(p) -> int:
    if p in (GD_PREC_F32, "f32", "fp32", "float32"):
        return GD_PREC_F32
    if p in (GD_PREC_F64, "f64", "fp64", "float64"):
        return GD_PREC_F64
    raise ValueError(f"unknown precision {p!r}")


class Complex:
    """A receptor + positioned ligand resident on the GPU (gd_complex)."""

    def __init__(self, receptor: Molecule, ligand: Molecule, restraint_pairs: Sequence[Tuple[int, int]] = (),
                 weights: EnergyWeights = EnergyWeights(), ctx: Optional[Context] = None):
        self.ctx = ctx or default_context()
        self.lib = self.ctx.lib
        self.receptor, self.ligand = receptor, ligand
        self._r, self._l = PackedAtoms(receptor), PackedAtoms(ligand)
        pairs = np.ascontiguousarray(np.asarray(list(restraint_pairs), dtype=np.int32).reshape(-1, 2))
        w = _lib.GdWeights(weights.vdw, weights.elec, weights.desolv, weights.air)
        h = C.c_void_p()
        self.ctx.check(self.lib.gd_complex_create(self.ctx.h, C.byref(self._r.s), C.byref(self._l.s),
                                                  ptr(pairs) if pairs.size else None, pairs.shape[0],
                                                  C.byref(w), C.byref(h)))
        self.h = h

    @property
    def num_restraints(self) -> int:
        return int(self.lib.gd_complex_num_restraints(self.h))

    def close(self):
        if getattr(self, "h", None):
            self.lib.gd_complex_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def score_poses(self, genes, precision=GD_PREC_F64) -> np.ndarray:
        """Energies of n poses (genes n x 6) as a structured array with the
        fields fitness, vdw, elec, desolv, air, restraint_penalty."""
        g = np.ascontiguousarray(genes, dtype=np.float64).reshape(-1, 6)
        out = np.zeros(g.shape[0], dtype=POSE_ENERGY_DTYPE)
        self.ctx.check(self.lib.gd_score_poses(self.h, ptr(g), g.shape[0], _prec(precision), ptr(out)))
        return out

    def score_models(self, xyz, precision=GD_PREC_F64) -> np.ndarray:
        """Energies of ligand coordinate sets given as is (n x n_lig x 3)."""
        x = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, len(self.ligand), 3)
        out = np.zeros(x.shape[0], dtype=POSE_ENERGY_DTYPE)
        self.ctx.check(self.lib.gd_score_models(self.h, ptr(x), x.shape[0], _prec(precision), ptr(out)))
        return out

    def pose_contacts(self, genes) -> List[np.ndarray]:
        g = np.ascontiguousarray(genes, dtype=np.float64).reshape(-1, 6)
        n = g.shape[0]
        offs = np.zeros(n + 1, dtype=np.int64)
        cap = max(1 << 16, 1024 * n)  # a second call only when poses average over 1,024 contacts
        for _ in range(2):
            keys = np.zeros(cap, dtype=np.int64)
            st = self.lib.gd_pose_contacts(self.h, ptr(g), n, ptr(keys), cap, ptr(offs))
            if st == _lib.GD_ERR_CAPACITY:
                cap = int(offs[n])
                continue
            self.ctx.check(st)
            break
        return [keys[offs[i]:offs[i + 1]].copy() for i in range(n)]

    def cluster(self, genes, config: ClusteringConfig = ClusteringConfig()) -> List[ClusterResult]:
        g = np.ascontiguousarray(genes, dtype=np.float64).reshape(-1, 6)
        n = g.shape[0]
        centers, sizes, members = (np.zeros(max(n, 1), np.int32) for _ in range(3))
        k = C.c_int32(0)
        cfg = config.c()
        self.ctx.check(self.lib.gd_cluster(self.h, ptr(g), n, C.byref(cfg), C.byref(k), ptr(centers), ptr(sizes),
                                           ptr(members)))
        return _results(k.value, centers, sizes, members)


@dataclass
class Metrics:
    """src/evaluator.rs:29-47"""
    rmsd: float
    irmsd: float
    fnat: float
    dockq: float

    def rank(self) -> str:
        return "High" if self.dockq >= 0.8 else "Medium" if self.dockq >= 0.5 else "Low"


class Evaluator:
    """DockQ, L-RMSD, i-RMSD and Fnat of poses of a complex's ligand against a
    reference ligand structure (gd_evaluator): Evaluator::new(receptor,
    reference) with the receptor of ``complex``."""

    def __init__(self, complex: Complex, reference: Molecule):
        self.cx, self.ctx, self.lib = complex, complex.ctx, complex.lib
        self._ref = PackedAtoms(reference)
        self._names = [pack_names(m.name) for m in (complex.receptor, complex.ligand, reference)]
        h = C.c_void_p()
        self.ctx.check(self.lib.gd_evaluator_create(complex.h, C.byref(self._ref.s), *[ptr(n) for n in self._names],
                                                    C.byref(h)))
        self.h = h

    def eval_metrics(self, genes) -> np.ndarray:
        """Metrics of n poses (genes n x 6) as a structured array with the
        fields rmsd, irmsd, fnat, dockq."""
        g = np.ascontiguousarray(genes, dtype=np.float64).reshape(-1, 6)
        out = np.zeros(g.shape[0], dtype=DOCK_METRICS_DTYPE)
        self.ctx.check(self.lib.gd_evaluate_poses(self.h, ptr(g), g.shape[0], ptr(out)))
        return out

    COUNT_NAMES = ("receptor_interface_residues", "reference_interface_residues", "native_contacts",
                   "ligand_atoms_read", "lrmsd_pairs", "irmsd_pairs", "contact_pairs_tested")

    def counts(self) -> dict:
        c = np.zeros(len(self.COUNT_NAMES), dtype=np.int64)
        self.ctx.check(self.lib.gd_evaluator_counts(self.h, ptr(c)))
        return dict(zip(self.COUNT_NAMES, c.tolist()))

    def eval_frames_device(self, d_frames: int, n: int, d_out: int, stream: Optional[int] = None):
        """gd_evaluate_frames_device: device pointers of n pose frames and of
        n metrics records; asynchronous on ``stream`` (a cudaStream_t)."""
        self.ctx.check(self.lib.gd_evaluate_frames_device(self.h, d_frames, n, d_out, stream))

    def calc_metrics(self, genes) -> Metrics:
        m = self.eval_metrics(np.asarray(genes, dtype=np.float64).reshape(1, 6))[0]
        return Metrics(*(float(m[k]) for k in DOCK_METRICS_DTYPE.names))

    def close(self):
        if getattr(self, "h", None):
            self.lib.gd_evaluator_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _results(k, centers, sizes, members) -> List[ClusterResult]:
    out, m = [], 0
    for c in range(k):
        s = int(sizes[c])
        out.append(ClusterResult(int(centers[c]), members[m:m + s].tolist(), s))
        m += s
    return out


def cluster_sets(sets: Sequence[np.ndarray], config: ClusteringConfig = ClusteringConfig(),
                 ctx: Optional[Context] = None) -> List[ClusterResult]:
    """cluster_structures on precomputed contact-key sets (FCC on the GPU)."""
    ctx = ctx or default_context()
    n = len(sets)
    offs = np.zeros(n + 1, dtype=np.int64)
    for i, s in enumerate(sets):
        offs[i + 1] = offs[i] + len(s)
    keys = np.ascontiguousarray(np.concatenate([np.asarray(s, np.int64) for s in sets]) if n else np.zeros(1, np.int64))
    if keys.size == 0:
        keys = np.zeros(1, np.int64)
    centers, sizes, members = (np.zeros(max(n, 1), np.int32) for _ in range(3))
    k = C.c_int32(0)
    cfg = config.c()
    ctx.check(ctx.lib.gd_cluster_sets(ctx.h, ptr(keys), ptr(offs), n, C.byref(cfg), C.byref(k), ptr(centers),
                                      ptr(sizes), ptr(members)))
    return _results(k.value, centers, sizes, members)


# -- reference-named energy functions (src/fitness.rs) -------------------------

def _one_shot(receptor, ligand, pairs=(), precision=GD_PREC_F64):
    cx = Complex(receptor, ligand, pairs)
    try:
        return cx.score_models(ligand.xyz()[None], precision)[0], cx.num_restraints
    finally:
        cx.close()


def vdw_energy(receptor: Molecule, ligand: Molecule) -> float:
    return float(_one_shot(receptor, ligand)[0]["vdw"])


def elec_energy(receptor: Molecule, ligand: Molecule) -> float:
    return float(_one_shot(receptor, ligand)[0]["elec"])


def desolv_energy(receptor: Molecule, ligand: Molecule) -> float:
    return float(_one_shot(receptor, ligand)[0]["desolv"])


def air_energy(restraint_pairs, receptor: Molecule, ligand: Molecule) -> float:
    return float(_one_shot(receptor, ligand, restraint_pairs)[0]["air"])


def satisfaction_ratio(restraint_pairs, receptor: Molecule, ligand: Molecule) -> float:
    e, k = _one_shot(receptor, ligand, restraint_pairs)
    return 0.0 if k == 0 else 1.0 - float(e["restraint_penalty"]) / k


@dataclass
class GaResult:
    genes: np.ndarray          # (jobs, pop, 6) final populations
    energies: np.ndarray       # (jobs, pop) structured energies of the final populations
    generations: np.ndarray    # (jobs,) generations evolved
    history: np.ndarray        # (jobs, max_generations) best fitness per generation
    hall_of_fame: Optional[List[np.ndarray]] = None  # per job, HOF_ENTRY_DTYPE records in the reference's order
    best_metrics: Optional[np.ndarray] = None  # (jobs, generations) DOCK_METRICS_DTYPE of each generation's best pose
    mean_dockq: Optional[np.ndarray] = None    # (jobs, generations) mean DockQ of each generation


def run_ga(complexes: Sequence[Complex], cfg=None, precision=GD_PREC_F32, use_graph: bool = True,
           ctx: Optional[Context] = None, hall_of_fame: bool = False,
           evaluators: Optional[Sequence[Optional["Evaluator"]]] = None) -> GaResult:
    """gdock's GA loop (src/commands/run.rs:381-531) for many jobs on the GPU;
    with ``hall_of_fame`` also each job's HallOfFame (src/commands/run.rs:77-213);
    with ``evaluators`` (one per job, None allowed) the DockQ metrics of every
    generation (src/commands/run.rs:388,449-451; NaN where not reached)."""
    ctx = ctx or complexes[0].ctx
    cfg = cfg or ga_default_cfg()
    J, n, G = len(complexes), cfg.pop_size, cfg.max_generations
    handles = (C.c_void_p * J)(*[c.h.value for c in complexes])
    genes = np.zeros((J, n, 6))
    energies = np.zeros((J, n), dtype=POSE_ENERGY_DTYPE)
    gens = np.zeros(J, np.int32)
    hist = np.zeros((J, max(G, 1)))
    hof = np.zeros((J, max(cfg.hof_max_size, 1)), dtype=HOF_ENTRY_DTYPE) if hall_of_fame else None
    hof_n = np.zeros(J, np.int32) if hall_of_fame else None
    best = mean = met = None
    if evaluators is not None:
        evh = (C.c_void_p * J)(*[e.h.value if e is not None else None for e in evaluators])
        best = np.full((J, max(G, 1)), np.nan, dtype=DOCK_METRICS_DTYPE)
        mean = np.full((J, max(G, 1)), np.nan)
        met = _lib.GdGaMetrics(C.cast(evh, C.c_void_p), ptr(best), ptr(mean))
    ctx.check(ctx.lib.gd_ga_run(ctx.h, C.cast(handles, C.c_void_p), J, C.byref(cfg), _prec(precision),
                                1 if use_graph else 0, ptr(genes), ptr(energies), ptr(gens), ptr(hist),
                                ptr(hof) if hall_of_fame else None, ptr(hof_n) if hall_of_fame else None,
                                C.byref(met) if met is not None else None))
    hl = [hof[j, :hof_n[j]].copy() for j in range(J)] if hall_of_fame else None
    return GaResult(genes, energies, gens, hist[:, :G], hl, best[:, :G] if best is not None else None,
                    mean[:, :G] if mean is not None else None)


class Server:
    """The serving loop (gd_server): docking jobs admitted into resident slots
    by HBM budget and advanced together, one generation per tick."""

    def __init__(self, ctx: Optional[Context] = None, max_slots: int = 64, hbm_budget: int = 0, ga=None,
                 precision=GD_PREC_F32):
        self.ctx = ctx or default_context()
        self.lib = self.ctx.lib
        cfg = _lib.GdServerCfg()
        self.lib.gd_server_default_cfg(C.byref(cfg))
        cfg.max_slots = max_slots
        cfg.hbm_budget = hbm_budget
        if ga is not None:
            cfg.ga = ga
        cfg.precision = _prec(precision)
        self.cfg = cfg
        h = C.c_void_p()
        self.ctx.check(self.lib.gd_server_create(self.ctx.h, C.byref(cfg), C.byref(h)))
        self.h = h

    def submit(self, receptor: Molecule, ligand: Molecule, restraint_pairs=(), seed: int = 42,
               weights: EnergyWeights = EnergyWeights()) -> int:
        r, l = PackedAtoms(receptor), PackedAtoms(ligand)
        pairs = np.ascontiguousarray(np.asarray(list(restraint_pairs), dtype=np.int32).reshape(-1, 2))
        w = _lib.GdWeights(weights.vdw, weights.elec, weights.desolv, weights.air)
        jid = C.c_int64()
        self.ctx.check(self.lib.gd_server_submit(self.h, C.byref(r.s), C.byref(l.s), ptr(pairs) if pairs.size else None,
                                                 pairs.shape[0], C.byref(w), seed, C.byref(jid)))
        return jid.value

    def step(self) -> int:
        a = C.c_int32()
        self.ctx.check(self.lib.gd_server_step(self.h, C.byref(a)))
        return a.value

    def start(self):
        self.ctx.check(self.lib.gd_server_start(self.h))

    def stop(self):
        self.ctx.check(self.lib.gd_server_stop(self.h))

    def wait(self, job: int, timeout_s: float = 600.0) -> int:
        st = C.c_int32()
        self.lib.gd_server_wait(self.h, job, timeout_s, C.byref(st))
        return st.value

    def result(self, job: int):
        n, G = self.cfg.ga.pop_size, max(self.cfg.ga.max_generations, 1)
        res = _lib.GdJobResult()
        genes = np.zeros((n, 6))
        energies = np.zeros(n, dtype=POSE_ENERGY_DTYPE)
        hist = np.zeros(G)
        self.ctx.check(self.lib.gd_server_result(self.h, job, C.byref(res), ptr(genes), ptr(energies), ptr(hist)))
        return res, genes, energies, hist[: self.cfg.ga.max_generations]

    def hall_of_fame(self, job: int) -> np.ndarray:
        """The finished job's Hall of Fame (HOF_ENTRY_DTYPE records)."""
        cap = max(self.cfg.ga.hof_max_size, 1)
        out = np.zeros(cap, dtype=HOF_ENTRY_DTYPE)
        k = C.c_int32(0)
        self.ctx.check(self.lib.gd_server_hall_of_fame(self.h, job, ptr(out), cap, C.byref(k)))
        return out[:k.value].copy()

    def release(self, job: int):
        self.ctx.check(self.lib.gd_server_release(self.h, job))

    def stats(self) -> "_lib.GdServerStats":
        s = _lib.GdServerStats()
        self.ctx.check(self.lib.gd_server_get_stats(self.h, C.byref(s)))
        return s

    def close(self):
        if getattr(self, "h", None):
            self.lib.gd_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
