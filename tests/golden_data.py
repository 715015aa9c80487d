"""Molecules and expected outputs from tests/golden/*.npz (see make_golden.py)."""
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"


class GoldenMol:
    """The atom arrays gd.Complex and the oracle read, from a fixture."""

    def __init__(self, d, prefix):
        g = lambda k: d[f"{prefix}_{k}"]
        self.x, self.y, self.z = (np.ascontiguousarray(g(k), np.float64) for k in ("x", "y", "z"))
        self.epsilon, self.rmin2 = g("epsilon").astype(np.float64), g("rmin2").astype(np.float64)
        self.charge, self.vdw_radius = g("charge").astype(np.float64), g("vdw_radius").astype(np.float64)
        self.serial, self.resseq = g("serial").astype(np.int32), g("resseq").astype(np.int16)
        self.chain_code, self.element_class = g("chain").astype(np.uint8), g("element").astype(np.uint8)
        self.is_ca = g("is_ca").astype(np.uint8)
        self.name = list(g("name"))
        self.chainid = [chr(c) for c in self.chain_code.tolist()]

    def __len__(self):
        return int(self.x.shape[0])

    def xyz(self):
        return np.stack([self.x, self.y, self.z], axis=1)


def load(name):
    d = np.load(GOLDEN / name)
    return d, GoldenMol(d, "rec"), GoldenMol(d, "lig")


def cluster_list(d):
    out, m = [], 0
    for c, s in zip(d["cluster_centers"].tolist(), d["cluster_sizes"].tolist()):
        out.append((c, d["cluster_members"][m:m + s].tolist()))
        m += s
    return out


def contact_sets(d):
    o, k = d["contact_offsets"], d["contact_keys"]
    return [k[o[i]:o[i + 1]] for i in range(len(o) - 1)]
