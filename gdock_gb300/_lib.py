"""ctypes bindings of libgdock_gb300.so (the C ABI in include/gdock_gb300.h).

The shared library is built in-tree (``gdock_gb300/_build``); loading fails
loudly when it is missing or when no CUDA device is present — there is no
CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "_build" / "libgdock_gb300.so"
LIB_DEBUG_PATH = Path(__file__).resolve().parent / "_build" / "libgdock_gb300_debug.so"
# GD_LIBRARY=debug selects the debug variant (kernel index checks compiled in)
DEBUG_LIBRARY = os.environ.get("GD_LIBRARY", "") == "debug"

GD_OK, GD_ERR_INVALID_ARG, GD_ERR_OOM, GD_ERR_CUDA, GD_ERR_TIMEOUT, GD_ERR_CAPACITY, GD_ERR_STATE = range(7)
GD_PREC_F64, GD_PREC_F32 = 0, 1

# every symbol the header declares (checked by the CPU test suite)
EXPORTS = (
    "gd_abi_version", "gd_status_string", "gd_context_create", "gd_context_destroy", "gd_last_error",
    "gd_context_bytes_in_use", "gd_complex_create", "gd_complex_destroy", "gd_complex_num_restraints",
    "gd_complex_set_weights", "gd_make_frames", "gd_score_poses", "gd_score_frames_device", "gd_sync",
    "gd_score_models", "gd_pose_contacts", "gd_cluster", "gd_cluster_sets", "gd_context_set_tuning",
    "gd_context_get_tuning", "gd_score_frames_device_noalloc", "gd_ga_default_cfg", "gd_ga_draw", "gd_ga_run",
    "gd_server_default_cfg", "gd_server_create", "gd_server_destroy", "gd_server_submit", "gd_server_step",
    "gd_server_start", "gd_server_stop", "gd_server_wait", "gd_server_result", "gd_server_release",
    "gd_server_get_stats", "gd_autotune_f32", "gd_evaluator_create", "gd_evaluator_destroy",
    "gd_evaluate_poses", "gd_evaluate_frames_device", "gd_evaluator_counts", "gd_server_hall_of_fame",
)
# candidates of gd_autotune_f32, in its order: (GD_TUNE_F32_SLOTS, GD_TUNE_SPLIT)
AUTOTUNE_CANDIDATES = ((16 + 4, 1), (64 + 2, 1), (64 + 4, 1), (256 + 64 + 2, 1), (256 + 64 + 4, 1), (256 + 64 + 4, 2))
GD_JOB_QUEUED, GD_JOB_RUNNING, GD_JOB_DONE, GD_JOB_FAILED = range(4)
GD_TUNE_F32_SLOTS = 0
GD_TUNE_SPLIT = 1
GD_TUNE_FAULT = 2
GD_TUNE_FCC = 3
GD_TUNE_CONTACTS = 4
GD_TUNE_RPARTS = 5
GD_INFO_LAST_FCC = 16
GD_INFO_LAST_CONTACTS = 17


class GdAtoms(C.Structure):
    _fields_ = [("n", C.c_int32), ("x", C.c_void_p), ("y", C.c_void_p), ("z", C.c_void_p),
                ("epsilon", C.c_void_p), ("rmin2", C.c_void_p), ("charge", C.c_void_p),
                ("vdw_radius", C.c_void_p), ("serial", C.c_void_p), ("resseq", C.c_void_p),
                ("chain", C.c_void_p), ("element", C.c_void_p), ("is_ca", C.c_void_p)]


class GdGaMetrics(C.Structure):
    _fields_ = [("evaluators", C.c_void_p), ("best", C.c_void_p), ("mean_dockq", C.c_void_p)]


class GdWeights(C.Structure):
    _fields_ = [("vdw", C.c_double), ("elec", C.c_double), ("desolv", C.c_double), ("air", C.c_double)]


class GdClusterCfg(C.Structure):
    _fields_ = [("contact_distance", C.c_double), ("fcc_cutoff", C.c_double), ("strictness", C.c_double),
                ("min_cluster_size", C.c_int32)]


class GdGaCfg(C.Structure):
    _fields_ = [("pop_size", C.c_int32), ("elitism", C.c_int32), ("tournament_size", C.c_int32),
                ("crossover_rate", C.c_double), ("mutation_rate", C.c_double), ("max_displacement", C.c_double),
                ("rot_sigma", C.c_double), ("trans_sigma", C.c_double), ("max_generations", C.c_int32),
                ("early_stopping", C.c_int32), ("convergence_threshold", C.c_double),
                ("convergence_window", C.c_int32), ("seed", C.c_uint64), ("hof_max_size", C.c_int32),
                ("hof_top_k", C.c_int32)]


class GdServerCfg(C.Structure):
    _fields_ = [("max_slots", C.c_int32), ("hbm_budget", C.c_uint64), ("ga", GdGaCfg), ("precision", C.c_int32)]


class GdJobResult(C.Structure):
    _fields_ = [("status", C.c_int32), ("error", C.c_int32), ("generations", C.c_int32),
                ("latency_s", C.c_double), ("queue_s", C.c_double)]


class GdServerStats(C.Structure):
    _fields_ = [("completed", C.c_int64), ("queued", C.c_int64), ("resident", C.c_int64),
                ("generations_run", C.c_int64), ("poses_scored", C.c_int64), ("device_bytes", C.c_uint64),
                ("latency_p50_s", C.c_double), ("latency_p99_s", C.c_double), ("latency_max_s", C.c_double),
                ("gpu_busy_s", C.c_double), ("elapsed_s", C.c_double)]


POSE_ENERGY_DTYPE = np.dtype([(k, np.float64) for k in
                              ("fitness", "vdw", "elec", "desolv", "air", "restraint_penalty")])
POSE_FRAME_BYTES = 16 * 8
HOF_ENTRY_DTYPE = np.dtype([("genes", np.float64, (6,)), ("fitness", np.float64), ("generation", np.int32),
                            ("pad", np.int32)])
DOCK_METRICS_DTYPE = np.dtype([(k, np.float64) for k in ("rmsd", "irmsd", "fnat", "dockq")])


def pack_names(names) -> np.ndarray:
    """Trimmed atom names packed little-endian into one uint32 each (byte k =
    character k, zero-padded), as gd_evaluator_create takes them."""
    out = np.zeros(len(names), dtype=np.uint32)
    for i, n in enumerate(names):
        b = n.strip().encode("ascii")
        if len(b) > 4:
            raise ValueError(f"atom name {n!r} is longer than 4 characters")
        out[i] = int.from_bytes(b.ljust(4, b"\0"), "little")
    return out

_lib = None


class GdError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"gdock_gb300 error {status}: {msg}")
        self.status = status


def load(path: Path = None):
    """Load the library (building it first if the build is missing or stale);
    the debug variant when GD_LIBRARY=debug."""
    global _lib
    if _lib is not None:
        return _lib
    from . import build as _build
    _build.build(debug=DEBUG_LIBRARY)
    lib = C.CDLL(str(path or (LIB_DEBUG_PATH if DEBUG_LIBRARY else LIB_PATH)))
    vp, i32, i64, d = C.c_void_p, C.c_int32, C.c_int64, C.c_double
    sigs = {
        "gd_abi_version": ([], i32),
        "gd_status_string": ([C.c_int], C.c_char_p),
        "gd_context_create": ([i32, C.c_uint64, C.POINTER(vp)], C.c_int),
        "gd_context_destroy": ([vp], C.c_int),
        "gd_last_error": ([vp], C.c_char_p),
        "gd_context_bytes_in_use": ([vp], C.c_uint64),
        "gd_complex_create": ([vp, C.POINTER(GdAtoms), C.POINTER(GdAtoms), vp, i32, C.POINTER(GdWeights),
                               C.POINTER(vp)], C.c_int),
        "gd_complex_destroy": ([vp], C.c_int),
        "gd_complex_num_restraints": ([vp], i32),
        "gd_complex_set_weights": ([vp, C.POINTER(GdWeights)], C.c_int),
        "gd_make_frames": ([vp, i32, vp], C.c_int),
        "gd_score_poses": ([vp, vp, i32, C.c_int, vp], C.c_int),
        "gd_score_frames_device": ([vp, vp, i32, C.c_int, d, vp, vp], C.c_int),
        "gd_sync": ([vp], C.c_int),
        "gd_score_models": ([vp, vp, i32, C.c_int, vp], C.c_int),
        "gd_pose_contacts": ([vp, vp, i32, vp, i64, vp], C.c_int),
        "gd_cluster": ([vp, vp, i32, C.POINTER(GdClusterCfg), C.POINTER(i32), vp, vp, vp], C.c_int),
        "gd_cluster_sets": ([vp, vp, vp, i32, C.POINTER(GdClusterCfg), C.POINTER(i32), vp, vp, vp], C.c_int),
        "gd_context_set_tuning": ([vp, i32, i32], C.c_int),
        "gd_context_get_tuning": ([vp, i32], i32),
        "gd_score_frames_device_noalloc": ([vp, vp, i32, d, vp, vp], C.c_int),
        "gd_ga_default_cfg": ([C.POINTER(GdGaCfg)], C.c_int),
        "gd_ga_draw": ([C.POINTER(GdGaCfg), C.c_uint64, i32, vp, vp, vp, vp, vp, vp], C.c_int),
        "gd_ga_run": ([vp, vp, i32, C.POINTER(GdGaCfg), C.c_int, i32, vp, vp, vp, vp, vp, vp, C.POINTER(GdGaMetrics)],
                      C.c_int),
        "gd_server_default_cfg": ([C.POINTER(GdServerCfg)], C.c_int),
        "gd_server_create": ([vp, C.POINTER(GdServerCfg), C.POINTER(vp)], C.c_int),
        "gd_server_destroy": ([vp], C.c_int),
        "gd_server_submit": ([vp, C.POINTER(GdAtoms), C.POINTER(GdAtoms), vp, i32, C.POINTER(GdWeights),
                              C.c_uint64, C.POINTER(i64)], C.c_int),
        "gd_server_step": ([vp, C.POINTER(i32)], C.c_int),
        "gd_server_start": ([vp], C.c_int),
        "gd_server_stop": ([vp], C.c_int),
        "gd_server_wait": ([vp, i64, d, C.POINTER(i32)], C.c_int),
        "gd_server_result": ([vp, i64, C.POINTER(GdJobResult), vp, vp, vp], C.c_int),
        "gd_server_release": ([vp, i64], C.c_int),
        "gd_server_get_stats": ([vp, C.POINTER(GdServerStats)], C.c_int),
        "gd_autotune_f32": ([vp, vp, i32, d, vp, vp, vp, C.POINTER(i32)], C.c_int),
        "gd_evaluator_create": ([vp, C.POINTER(GdAtoms), vp, vp, vp, C.POINTER(vp)], C.c_int),
        "gd_evaluator_destroy": ([vp], C.c_int),
        "gd_evaluate_poses": ([vp, vp, i32, vp], C.c_int),
        "gd_evaluate_frames_device": ([vp, vp, i32, vp, vp], C.c_int),
        "gd_evaluator_counts": ([vp, vp], C.c_int),
        "gd_server_hall_of_fame": ([vp, i64, vp, i32, C.POINTER(i32)], C.c_int),
    }
    for name, (args, res) in sigs.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res
    _lib = lib
    return lib


def ptr(a: np.ndarray) -> int:
    return a.ctypes.data


class Context:
    """One CUDA device context of the library."""

    def __init__(self, device: int = 0, hbm_budget_bytes: int = 0):
        self.lib = load()
        h = C.c_void_p()
        st = self.lib.gd_context_create(device, hbm_budget_bytes, C.byref(h))
        if st != GD_OK:
            raise GdError(st, f"gd_context_create failed ({self.lib.gd_status_string(st).decode()}); "
                              "a CUDA device is required")
        self.h = h

    def check(self, st: int):
        if st != GD_OK:
            raise GdError(st, self.lib.gd_last_error(self.h).decode())

    def close(self):
        if self.h:
            self.lib.gd_context_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def sync(self):
        self.check(self.lib.gd_sync(self.h))

    def set_tuning(self, knob: int, value: int):
        self.check(self.lib.gd_context_set_tuning(self.h, knob, value))

    def get_tuning(self, knob: int) -> int:
        """A knob's value, or a read-only GD_INFO_* value."""
        return int(self.lib.gd_context_get_tuning(self.h, knob))

    @property
    def bytes_in_use(self) -> int:
        return int(self.lib.gd_context_bytes_in_use(self.h))


class PackedAtoms:
    """gd_atoms view of a pdb.Molecule; keeps the numpy buffers alive."""

    def __init__(self, mol):
        c = np.ascontiguousarray
        self.bufs = [c(mol.x, np.float64), c(mol.y, np.float64), c(mol.z, np.float64),
                     c(mol.epsilon, np.float64), c(mol.rmin2, np.float64), c(mol.charge, np.float64),
                     c(mol.vdw_radius, np.float64), c(mol.serial, np.int32), c(mol.resseq, np.int16),
                     c(mol.chain_code, np.uint8), c(mol.element_class, np.uint8), c(mol.is_ca, np.uint8)]
        self.s = GdAtoms(len(mol), *[ptr(b) for b in self.bufs])
        self.s._keep = self.bufs  # the struct holds raw addresses: keep the buffers alive with it


def make_frames(genes: np.ndarray) -> np.ndarray:
    """Pose frames (n x 16 doubles) of n x 6 genes, computed by the library."""
    lib = load()
    g = np.ascontiguousarray(genes, dtype=np.float64).reshape(-1, 6)
    out = np.zeros((g.shape[0], 16))
    st = lib.gd_make_frames(ptr(g), g.shape[0], ptr(out))
    if st != GD_OK:
        raise GdError(st, "gd_make_frames")
    return out


def ga_default_cfg(**overrides) -> GdGaCfg:
    c = GdGaCfg()
    load().gd_ga_default_cfg(C.byref(c))
    for k, v in overrides.items():
        setattr(c, k, v)
    return c


def ga_draw(cfg: GdGaCfg, seed: int, generations: int) -> dict:
    """The host draws of one GA job (initial genes and per-generation randoms)."""
    n = cfg.pop_size
    m = 2 * (n // 2)
    G = max(generations, 0)
    out = {"init": np.zeros((n, 6)), "tour": np.zeros((G, n * cfg.tournament_size), np.int32),
           "perm": np.zeros((G, n), np.int32), "cross_u": np.zeros((G, 6 * (n // 2))),
           "mut_u": np.zeros((G, 6 * m)), "mut_z": np.zeros((G, 6 * m))}
    st = load().gd_ga_draw(C.byref(cfg), seed, G, *[ptr(out[k]) if out[k].size else None for k in
                                                     ("init", "tour", "perm", "cross_u", "mut_u", "mut_z")])
    if st != GD_OK:
        raise GdError(st, "gd_ga_draw")
    return out
