"""ctypes front end of the CPU oracle (test infrastructure only).

Tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py``
load this module to check or time against; the GPU product path never
imports it.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess
from pathlib import Path

import numpy as np

_HERE = Path(__file__).resolve().parent
_LIB_PATH = _HERE / "_build" / "libgd_oracle.so"
_lib = None


def build(force: bool = False) -> Path:
    src = [_HERE / "gd_oracle.c", _HERE / "gd_oracle.h"]
    if force or not _LIB_PATH.exists() or any(s.stat().st_mtime > _LIB_PATH.stat().st_mtime for s in src):
        subprocess.run(["make", "-s", "-C", str(_HERE)], check=True)
    return _LIB_PATH


class OrcMol(C.Structure):
    _fields_ = [("n", C.c_int32),
                ("x", C.c_void_p), ("y", C.c_void_p), ("z", C.c_void_p),
                ("epsilon", C.c_void_p), ("rmin2", C.c_void_p), ("charge", C.c_void_p),
                ("vdw_radius", C.c_void_p), ("serial", C.c_void_p), ("resseq", C.c_void_p),
                ("chain", C.c_void_p), ("element", C.c_void_p), ("is_ca", C.c_void_p)]


class OrcWeights(C.Structure):
    _fields_ = [("vdw", C.c_double), ("elec", C.c_double), ("desolv", C.c_double), ("air", C.c_double)]


ENERGY_FIELDS = ("fitness", "vdw", "elec", "desolv", "air", "restraint_penalty")
DEFAULT_WEIGHTS = (0.4, 0.05, 3.4, 1.0)  # src/constants.rs:22-25


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(str(_LIB_PATH))
        P = C.POINTER
        _lib.orc_vdw_energy.restype = C.c_double
        _lib.orc_elec_energy.restype = C.c_double
        _lib.orc_desolv_energy.restype = C.c_double
        _lib.orc_air_energy.restype = C.c_double
        _lib.orc_satisfaction_ratio.restype = C.c_double
        _lib.orc_count_restraints.restype = C.c_int32
        _lib.orc_contacts.restype = C.c_int32
        _lib.orc_pose_contacts.restype = C.c_int32
        _lib.orc_cluster.restype = C.c_int32
        for f in ("orc_vdw_energy", "orc_elec_energy", "orc_desolv_energy"):
            getattr(_lib, f).argtypes = [P(OrcMol), P(OrcMol)]
    return _lib


class _Packed:
    """Keeps the numpy buffers of an OrcMol alive."""

    def __init__(self, mol, x=None, y=None, z=None):
        c = np.ascontiguousarray
        self.bufs = [
            c(mol.x if x is None else x, dtype=np.float64), c(mol.y if y is None else y, dtype=np.float64),
            c(mol.z if z is None else z, dtype=np.float64), c(mol.epsilon, dtype=np.float64),
            c(mol.rmin2, dtype=np.float64), c(mol.charge, dtype=np.float64),
            c(mol.vdw_radius, dtype=np.float64), c(mol.serial, dtype=np.int32),
            c(mol.resseq, dtype=np.int16), c(mol.chain_code, dtype=np.uint8),
            c(mol.element_class, dtype=np.uint8), c(mol.is_ca, dtype=np.uint8)]
        self.s = OrcMol(len(mol), *[b.ctypes.data for b in self.bufs])
        # the struct holds raw addresses only: tie the buffers' lifetime to it,
        # so that a byref() of a temporary keeps them alive for the call
        self.s._keep = self.bufs

    @property
    def ref(self):
        return C.byref(self.s)


def pack(mol, x=None, y=None, z=None) -> _Packed:
    return _Packed(mol, x, y, z)


def _pairs(pairs):
    a = np.ascontiguousarray(np.asarray(pairs, dtype=np.int32).reshape(-1, 2))
    return a, a.shape[0]


def vdw_energy(rec, lig) -> float:
    return lib().orc_vdw_energy(pack(rec).ref, pack(lig).ref)


def elec_energy(rec, lig) -> float:
    return lib().orc_elec_energy(pack(rec).ref, pack(lig).ref)


def desolv_energy(rec, lig) -> float:
    return lib().orc_desolv_energy(pack(rec).ref, pack(lig).ref)


def air_energy(pairs, rec, lig) -> float:
    a, k = _pairs(pairs)
    return lib().orc_air_energy(a.ctypes.data_as(C.c_void_p), C.c_int32(k), pack(rec).ref, pack(lig).ref)


def satisfaction_ratio(pairs, rec, lig) -> float:
    a, k = _pairs(pairs)
    return lib().orc_satisfaction_ratio(a.ctypes.data_as(C.c_void_p), C.c_int32(k), pack(rec).ref, pack(lig).ref)


def kept_restraints(pairs, rec, lig) -> np.ndarray:
    a, k = _pairs(pairs)
    out = np.zeros_like(a)
    m = lib().orc_count_restraints(a.ctypes.data_as(C.c_void_p), C.c_int32(k), pack(rec).ref,
                                   pack(lig).ref, out.ctypes.data_as(C.c_void_p))
    return out[:m].copy()


def apply_genes(lig, genes):
    n = len(lig)
    x, y, z = np.empty(n), np.empty(n), np.empty(n)
    g = np.ascontiguousarray(genes, dtype=np.float64)
    lib().orc_apply_genes(pack(lig).ref, g.ctypes.data_as(C.c_void_p), x.ctypes.data_as(C.c_void_p),
                          y.ctypes.data_as(C.c_void_p), z.ctypes.data_as(C.c_void_p))
    return x, y, z


def score_poses(rec, lig, pairs, genes, weights=DEFAULT_WEIGHTS, nthreads=None) -> np.ndarray:
    """(n, 6) array of fitness, vdw, elec, desolv, air, restraint_penalty.
    `pairs` are the restraint residue pairs; the ones whose CAs are missing
    are dropped first, as gdock does when it builds restraints."""
    kept = kept_restraints(pairs, rec, lig)
    g = np.ascontiguousarray(np.asarray(genes, dtype=np.float64).reshape(-1, 6))
    out = np.zeros((g.shape[0], 6))
    w = OrcWeights(*weights)
    pr, pl = pack(rec), pack(lig)
    lib().orc_score_poses(pr.ref, pl.ref, kept.ctypes.data_as(C.c_void_p), C.c_int32(kept.shape[0]),
                          C.byref(w), g.ctypes.data_as(C.c_void_p), C.c_int32(g.shape[0]),
                          out.ctypes.data_as(C.c_void_p), C.c_int32(nthreads or os.cpu_count() or 1))
    return out


def score_models(rec, lig, pairs, xyz, weights=DEFAULT_WEIGHTS, nthreads=None) -> np.ndarray:
    kept = kept_restraints(pairs, rec, lig)
    x = np.ascontiguousarray(np.asarray(xyz, dtype=np.float64).reshape(-1, len(lig), 3))
    out = np.zeros((x.shape[0], 6))
    w = OrcWeights(*weights)
    pr, pl = pack(rec), pack(lig)
    lib().orc_score_models(pr.ref, pl.ref, kept.ctypes.data_as(C.c_void_p), C.c_int32(kept.shape[0]),
                           C.byref(w), x.ctypes.data_as(C.c_void_p), C.c_int32(x.shape[0]),
                           out.ctypes.data_as(C.c_void_p), C.c_int32(nthreads or os.cpu_count() or 1))
    return out


def contacts(mol, cutoff=5.0) -> np.ndarray:
    cap = 1 << 20
    keys = np.zeros(cap, dtype=np.int64)
    n = lib().orc_contacts(pack(mol).ref, C.c_double(cutoff), keys.ctypes.data_as(C.c_void_p), C.c_int32(cap))
    return keys[: min(n, cap)].copy()


def pose_contacts(rec, lig, genes, cutoff=5.0) -> np.ndarray:
    cap = 1 << 20
    keys = np.zeros(cap, dtype=np.int64)
    g = np.ascontiguousarray(genes, dtype=np.float64)
    n = lib().orc_pose_contacts(pack(rec).ref, pack(lig).ref, g.ctypes.data_as(C.c_void_p), C.c_double(cutoff),
                                keys.ctypes.data_as(C.c_void_p), C.c_int32(cap))
    return keys[: min(n, cap)].copy()


def pose_contacts_many(rec, lig, genes, cutoff=5.0, nthreads=None):
    """pose_contacts of every gene vector, on a pool of host threads (the C
    restatement releases the interpreter lock while it runs)."""
    from concurrent.futures import ThreadPoolExecutor
    g = np.asarray(genes, dtype=np.float64).reshape(-1, 6)
    with ThreadPoolExecutor(max_workers=nthreads or os.cpu_count() or 1) as ex:
        return list(ex.map(lambda row: pose_contacts(rec, lig, row, cutoff), g))


def _flatten_sets(sets):
    offs = np.zeros(len(sets) + 1, dtype=np.int64)
    for i, s in enumerate(sets):
        offs[i + 1] = offs[i] + len(s)
    keys = np.concatenate([np.asarray(s, dtype=np.int64) for s in sets]) if sets else np.zeros(0, np.int64)
    return np.ascontiguousarray(keys), offs


def pairwise_fcc(sets):
    keys, offs = _flatten_sets(sets)
    n = len(sets)
    f, fv = np.zeros((n, n)), np.zeros((n, n))
    lib().orc_pairwise_fcc(keys.ctypes.data_as(C.c_void_p), offs.ctypes.data_as(C.c_void_p), C.c_int32(n),
                           f.ctypes.data_as(C.c_void_p), fv.ctypes.data_as(C.c_void_p))
    return f, fv


def cluster(sets, fcc_cutoff=0.60, strictness=0.75, min_size=4):
    """[(center, [members...]), ...] in gdock's output order."""
    keys, offs = _flatten_sets(sets)
    n = len(sets)
    centers = np.zeros(max(n, 1), np.int32)
    sizes = np.zeros(max(n, 1), np.int32)
    members = np.zeros(max(n, 1), np.int32)
    k = lib().orc_cluster(keys.ctypes.data_as(C.c_void_p), offs.ctypes.data_as(C.c_void_p), C.c_int32(n),
                          C.c_double(fcc_cutoff), C.c_double(strictness), C.c_int32(min_size),
                          centers.ctypes.data_as(C.c_void_p), sizes.ctypes.data_as(C.c_void_p),
                          members.ctypes.data_as(C.c_void_p))
    out, m = [], 0
    for c in range(k):
        out.append((int(centers[c]), members[m:m + sizes[c]].tolist()))
        m += int(sizes[c])
    return out


def contact_key(chain_a: str, res_a: int, chain_b: str, res_b: int) -> int:
    """Key of the contact string "cA rA cB rB" (smaller chain first)."""
    if chain_a > chain_b:
        chain_a, res_a, chain_b, res_b = chain_b, res_b, chain_a, res_a
    return (ord(chain_a) << 48) | ((res_a & 0xffff) << 32) | (ord(chain_b) << 16) | (res_b & 0xffff)


def evolve(genes, fitness, draws, g, elitism=5, tournament=3, crossover_rate=0.6, mutation_rate=0.1,
           max_displacement=50.0):
    """Population::evolve on explicit draws (generation g of a gd_ga_draw dict)."""
    genes = np.ascontiguousarray(genes, dtype=np.float64).reshape(-1, 6)
    fitness = np.ascontiguousarray(fitness, dtype=np.float64)
    n = genes.shape[0]
    m = 2 * (n // 2)
    go, fo = np.zeros((m, 6)), np.zeros(m)
    arrs = [np.ascontiguousarray(draws[k][g]) for k in ("tour", "perm", "cross_u", "mut_u", "mut_z")]
    lib().orc_evolve(C.c_int32(n), genes.ctypes.data_as(C.c_void_p), fitness.ctypes.data_as(C.c_void_p),
                     C.c_int32(elitism), arrs[0].ctypes.data_as(C.c_void_p), C.c_int32(tournament),
                     arrs[1].ctypes.data_as(C.c_void_p), arrs[2].ctypes.data_as(C.c_void_p),
                     C.c_double(crossover_rate), arrs[3].ctypes.data_as(C.c_void_p),
                     arrs[4].ctypes.data_as(C.c_void_p), C.c_double(mutation_rate), C.c_double(max_displacement),
                     go.ctypes.data_as(C.c_void_p), fo.ctypes.data_as(C.c_void_p))
    return go, fo


def ga_close_comparisons(f, tour, perm, tournament=3, tol=1e-9):
    """The fitness comparisons one generation's bookkeeping and evolve decide
    (first best of the generation, src/commands/run.rs:391-398; elitism's
    stable sort, src/population.rs:76-82; tournaments, :136-156; the stable
    sort of the offspring by carried fitness, :110-118), counted as
    (total, ties, close): ties = equal values (identical poses give identical
    energies in any implementation, so ties are resolved by index alike);
    close = unequal values decided by a relative margin below tol, the
    comparisons a difference of summation order in the energies could turn.
    Sorts count their adjacent pairs in sorted order."""
    f = np.asarray(f, dtype=np.float64)
    n = len(f)
    total = ties = close = 0

    def cmp(a, b):
        nonlocal total, ties, close
        total += 1
        if a == b:
            ties += 1
        elif abs(a - b) <= tol * max(abs(a), abs(b)):
            close += 1

    bi = 0
    for k in range(1, n):
        cmp(f[bi], f[k])
        if f[bi] > f[k]:
            bi = k
    srt = np.sort(f, kind="stable")
    for k in range(n - 1):
        cmp(srt[k], srt[k + 1])
    sel = []
    for k in range(n):
        best = int(tour[tournament * k])
        for t in range(1, tournament):
            q = int(tour[tournament * k + t])
            cmp(f[best], f[q])
            if f[best] > f[q]:
                best = q
        sel.append(best)
    m = 2 * (n // 2)
    carried = np.sort(np.array([f[sel[int(perm[i])]] for i in range(m)]), kind="stable")
    for k in range(m - 1):
        cmp(carried[k], carried[k + 1])
    return total, ties, close


class HallOfFame:
    """HallOfFame (src/commands/run.rs:75-215) restated: entries are
    (genes tuple, fitness, generation) in the reference's order."""

    def __init__(self, max_size=500, top_k=10, rot=0.2, trans=2.0):
        self.entries, self.max_size, self.top_k, self.rot, self.trans = [], max_size, top_k, rot, trans

    @staticmethod
    def angular_difference(a, b):  # src/commands/run.rs:162-171
        d = abs(a - b)
        return 2.0 * math.pi - d if d > math.pi else d

    def genes_are_similar(self, a, b):  # src/commands/run.rs:140-160
        for i in range(3):
            if self.angular_difference(a[i], b[i]) > self.rot:
                return False
        for i in range(3, 6):
            if abs(a[i] - b[i]) > self.trans:
                return False
        return True

    def try_add(self, genes, fitness, generation):  # src/commands/run.rs:101-127
        if len(genes) != 6:
            return False
        g = tuple(float(x) for x in genes)
        if any(self.genes_are_similar(g, e[0]) for e in self.entries):
            return False
        self.entries.append((g, float(fitness), int(generation)))
        if len(self.entries) > self.max_size:  # prune, :174-179 (a stable sort)
            self.entries.sort(key=lambda e: e[1])
            del self.entries[self.max_size:]
        return True

    def add_from_population(self, genes, fitness, generation):  # src/commands/run.rs:193-213
        order = sorted(range(len(fitness)), key=lambda k: fitness[k])  # stable
        added = 0
        for k in order:
            if added >= self.top_k:
                break
            if self.try_add(genes[k], fitness[k], generation):
                added += 1


def run_ga(rec, lig, pairs, cfg, draws, weights=DEFAULT_WEIGHTS, nthreads=None, hof=None, evaluator=None,
           metrics_out=None, close_out=None):
    """gdock's generation loop (src/commands/run.rs:381-531) on the CPU with
    explicit draws: returns final genes, final energies, generations, history;
    ``hof`` (a HallOfFame) is fed after every evaluation inside the loop
    (src/commands/run.rs:385); with ``evaluator`` (an Evaluator) the list
    ``metrics_out`` receives, per generation, the metrics (rmsd, irmsd, fnat,
    dockq) of the first best-fitness pose and the mean DockQ
    (src/commands/run.rs:388,449-451); ``close_out`` (a list) receives the
    (total, ties, close) fitness comparisons of every evolved generation
    (ga_close_comparisons)."""
    genes = draws["init"].copy()
    last_best, stagnant, history = None, 0, []
    gen = 0
    while True:
        e = score_poses(rec, lig, pairs, genes, weights, nthreads)
        if gen >= cfg.max_generations:
            return genes, e, gen, np.array(history)
        f = e[:, 0]
        if hof is not None:
            hof.add_from_population(genes, f, gen)
        if evaluator is not None:
            m = evaluator.eval_metrics(lig, genes)
            bi = 0
            for k in range(1, len(f)):
                if f[bi] > f[k]:
                    bi = k
            metrics_out.append((tuple(m[bi]), _seq_sum(m[:, 3]) / len(f)))
        best = f[int(np.argmin(f))]
        bi = 0
        for k in range(1, len(f)):
            if f[bi] > f[k]:
                bi = k
        best = f[bi]
        history.append(best)
        if gen > 0:
            imp = (last_best - best) / abs(last_best)
            stagnant = stagnant + 1 if imp < cfg.convergence_threshold else 0
        last_best = best
        if cfg.early_stopping and stagnant >= cfg.convergence_window:
            return genes, e, gen, np.array(history)
        if close_out is not None:
            close_out.append(ga_close_comparisons(f, draws["tour"][gen], draws["perm"][gen], cfg.tournament_size))
        genes, _ = evolve(genes, f, draws, gen, cfg.elitism, cfg.tournament_size, cfg.crossover_rate,
                          cfg.mutation_rate, cfg.max_displacement)
        gen += 1


# -- evaluator::Evaluator (src/evaluator.rs), restated on numpy ---------------

def _dist(ax, ay, az, bx, by, bz):
    """Atom::distance_to, sqrt((dx*dx + dy*dy) + dz*dz) (src/structure.rs:178-183)."""
    dx, dy, dz = ax - bx, ay - by, az - bz
    return np.sqrt(dx * dx + dy * dy + dz * dz)


def _seq_sum(v) -> float:
    """Left-to-right sum, as Iterator::sum (builtin sum() is compensated)."""
    s = 0.0
    for x in np.asarray(v, dtype=np.float64).tolist():
        s += x
    return s


def _atoms(mol, x=None, y=None, z=None):
    return (np.asarray(mol.x if x is None else x, np.float64), np.asarray(mol.y if y is None else y, np.float64),
            np.asarray(mol.z if z is None else z, np.float64), np.asarray(mol.resseq).astype(np.int64),
            list(mol.chainid), [n.strip() for n in mol.name])


def _contacts(a, b):
    """calculate_contacts (src/evaluator.rs:145-168): identities of the atom
    pairs at <= 5 A, receptor-major order, duplicates kept."""
    d = _dist(a[0][:, None], a[1][:, None], a[2][:, None], b[0][None, :], b[1][None, :], b[2][None, :])
    ii, jj = np.nonzero(d <= 5.0)
    return [(a[4][i], int(a[3][i]), a[5][i], b[4][j], int(b[3][j]), b[5][j]) for i, j in zip(ii.tolist(), jj.tolist())]


def _filter(m, keep):
    """structure::filter_by_resseq_vec (src/structure.rs:319-327)."""
    sel = np.array([int(r) in keep for r in m[3]], dtype=bool)
    idx = np.nonzero(sel)[0].tolist()
    return (m[0][sel], m[1][sel], m[2][sel], m[3][sel], [m[4][i] for i in idx], [m[5][i] for i in idx])


class Evaluator:
    """evaluator::Evaluator::new (src/evaluator.rs:50-66): interface residues
    (calculate_interface, :170-186), interface atoms and native contacts."""

    def __init__(self, rec, ref):
        self.rec, self.ref = _atoms(rec), _atoms(ref)
        r, f = self.rec, self.ref
        d = _dist(r[0][:, None], r[1][:, None], r[2][:, None], f[0][None, :], f[1][None, :], f[2][None, :])
        hit = d <= 5.0
        self.interface = (set(r[3][hit.any(axis=1)].tolist()), set(f[3][hit.any(axis=0)].tolist()))
        self.receptor_interface = _filter(r, self.interface[0])
        self.reference_interface = _filter(f, self.interface[1])
        self.native_contacts = _contacts(self.receptor_interface, self.reference_interface)
        self._native_set = set(self.native_contacts)

    def calc_rmsd(self, lig) -> float:
        """src/evaluator.rs:86-103 (a sum of distances, not of squares)."""
        n = len(self.ref[0])
        if n == 0:
            return 0.0
        k = min(len(lig[0]), n)
        d = _dist(lig[0][:k], lig[1][:k], lig[2][:k], self.ref[0][:k], self.ref[1][:k], self.ref[2][:k])
        return float(np.sqrt(_seq_sum(d) / n))

    def calc_irmsd(self, lig) -> float:
        """src/evaluator.rs:105-124"""
        t = _filter(lig, self.interface[1])
        ri = self.reference_interface
        n = len(ri[0])
        if n == 0:
            return 0.0
        k = min(len(t[0]), n)
        d = _dist(t[0][:k], t[1][:k], t[2][:k], ri[0][:k], ri[1][:k], ri[2][:k])
        return float(np.sqrt(_seq_sum(d) / n))

    def calc_fnat(self, lig) -> float:
        """src/evaluator.rs:126-143"""
        docked = _contacts(self.receptor_interface, _filter(lig, self.interface[1]))
        common = sum(1 for c in docked if c in self._native_set)
        if not self.native_contacts:
            return 0.0
        return common / len(self.native_contacts)

    def calc_metrics(self, lig_mol, x=None, y=None, z=None):
        """src/evaluator.rs:68-84: (rmsd, irmsd, fnat, dockq) of the ligand
        (optionally with moved coordinates x, y, z)."""
        lig = _atoms(lig_mol, x, y, z)
        fnat, irmsd, rmsd = self.calc_fnat(lig), self.calc_irmsd(lig), self.calc_rmsd(lig)
        a, b = irmsd / 1.5, rmsd / 8.5
        dockq = (fnat + 1.0 / (1.0 + a * a) + 1.0 / (1.0 + b * b)) / 3.0
        return rmsd, irmsd, fnat, dockq

    def eval_metrics(self, lig_mol, genes) -> np.ndarray:
        """Population::eval_metrics (src/population.rs:63-71): (n, 4) array."""
        g = np.ascontiguousarray(genes, dtype=np.float64).reshape(-1, 6)
        out = np.zeros((g.shape[0], 4))
        for i in range(g.shape[0]):
            out[i] = self.calc_metrics(lig_mol, *apply_genes(lig_mol, g[i]))
        return out
