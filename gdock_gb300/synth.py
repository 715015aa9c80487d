"""Seeded synthetic docking complexes and pose sets.

The reference's benchmark set (PPDB v5) is not available, so every workload
here is a synthetic complex built the same way each time from a seed:

* residue types uniform over the 20 standard amino acids, with the atom names
  of gdock's parameter table (histidine as ``HIS``, which the table maps);
* a C-alpha chain as a 3.8 A random walk confined to a globule whose radius
  is 12 A at 50 residues and grows with the cube root of the residue count;
* every other heavy atom of the residue placed 1.5-4 A from its C-alpha;
* receptor as chain A (serials 1..N_r), ligand as chain B (serials after
  the receptor's, unless ``overlap_serials`` asks for the 1-based numbering
  that makes gdock's equal-serial van der Waals skip fire);
* restraints pairing randomly chosen surface residues (largest C-alpha
  distance from the centroid).

Coordinates are rounded to the PDB's 3 decimals so that text files and
in-memory arrays are the same numbers on every machine.
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import List, Tuple

import numpy as np

from . import pdb as _pdb

STD20 = ["ALA", "ARG", "ASN", "ASP", "CYS", "GLN", "GLU", "GLY", "HIS", "ILE",
         "LEU", "LYS", "MET", "PHE", "PRO", "SER", "THR", "TRP", "TYR", "VAL"]
_BACKBONE = ["N", "CA", "C", "O"]


def _heavy_names(resname: str) -> List[str]:
    names = [a for a in _pdb.residue_atom_names(resname) if not a.startswith("H")]
    side = sorted(a for a in names if a not in _BACKBONE)
    return [a for a in _BACKBONE if a in names] + side


def globule_radius(n_res: int) -> float:
    return 12.0 * (n_res / 50.0) ** (1.0 / 3.0)


def _unit(rng) -> np.ndarray:
    v = rng.normal(size=3)
    return v / np.linalg.norm(v)


def _ca_walk(rng, n_res: int, radius: float) -> np.ndarray:
    ca = np.zeros((n_res, 3))
    ca[0] = _unit(rng) * radius * 0.3
    for k in range(1, n_res):
        best, best_r = None, None
        for _ in range(60):
            p = ca[k - 1] + 3.8 * _unit(rng)
            r = float(np.linalg.norm(p))
            if k > 1 and np.min(np.linalg.norm(ca[:k - 1] - p, axis=1)) < 3.0:
                continue
            if r <= radius:
                best = p
                break
            if best is None or r < best_r:
                best, best_r = p, r
        if best is None:
            best = ca[k - 1] + 3.8 * _unit(rng)
        ca[k] = best
    return ca


@dataclass
class Complex:
    receptor: _pdb.Molecule
    ligand: _pdb.Molecule
    restraint_pairs: List[Tuple[int, int]]
    seed: int

    def receptor_pdb(self) -> str:
        return _pdb.write_pdb_text(self.receptor)

    def ligand_pdb(self) -> str:
        return _pdb.write_pdb_text(self.ligand)


def make_chain(rng, n_res: int, chain: str, serial0: int, center) -> str:
    radius = globule_radius(n_res)
    ca = _ca_walk(rng, n_res, radius) + np.asarray(center, dtype=np.float64)
    res = rng.integers(0, len(STD20), size=n_res)
    lines = []
    serial = serial0
    for k in range(n_res):
        rn = STD20[int(res[k])]
        for name in _heavy_names(rn):
            if name == "CA":
                p = ca[k]
            else:
                p = ca[k] + rng.uniform(1.5, 4.0) * _unit(rng)
            lines.append(_pdb.atom_line(serial, name, rn, chain, k + 1,
                                        round(float(p[0]), 3), round(float(p[1]), 3),
                                        round(float(p[2]), 3), name[0]))
            serial += 1
    return "".join(lines)


def _surface_residues(mol: _pdb.Molecule) -> List[int]:
    ca = [i for i in range(len(mol)) if mol.name[i] == "CA"]
    c = np.array(mol.center_of_mass())
    d = [float(np.linalg.norm(mol.xyz()[i] - c)) for i in ca]
    order = np.argsort(-np.asarray(d), kind="stable")
    top = [int(mol.resseq[ca[i]]) for i in order[: max(1, len(ca) // 3)]]
    return top


def make_complex(n_rec_res: int, n_lig_res: int, n_restraints: int, seed: int,
                 overlap_serials: bool = False) -> Complex:
    rng = np.random.default_rng(seed)
    rec_txt = make_chain(rng, n_rec_res, "A", 1, (0.0, 0.0, 0.0))
    receptor = _pdb.read_pdb_text(rec_txt)[0]
    off = globule_radius(n_rec_res) + globule_radius(n_lig_res) + 6.0
    lig_txt = make_chain(rng, n_lig_res, "B", 1 if overlap_serials else len(receptor) + 1,
                         (off, 0.0, 0.0))
    ligand = _pdb.read_pdb_text(lig_txt)[0]
    rs, ls = _surface_residues(receptor), _surface_residues(ligand)
    k = min(n_restraints, len(rs), len(ls))
    ri = rng.choice(len(rs), size=k, replace=False)
    li = rng.choice(len(ls), size=k, replace=False)
    pairs = [(rs[int(a)], ls[int(b)]) for a, b in zip(ri, li)]
    return Complex(receptor, ligand, pairs, seed)


def random_genes(rng, n: int, max_displacement: float = 50.0) -> np.ndarray:
    """Genes drawn like a fresh chromosome: three angles in [0, 2*pi] and a
    displacement in [-50, 50]^3 (src/chromosome.rs:27-34)."""
    g = np.empty((n, 6))
    g[:, :3] = rng.uniform(0.0, 2.0 * math.pi, size=(n, 3))
    g[:, 3:] = rng.uniform(-max_displacement, max_displacement, size=(n, 3))
    return g


def quaternion_genes(rng, n: int, half_box: float = 20.0) -> np.ndarray:
    """Rotations uniform on SO(3) drawn as unit quaternions, expressed as the
    (alpha, beta, gamma) genes of gdock's rotation (src/structure.rs:96-103,
    which is Rz(alpha) Ry(beta) Rx(gamma)), and centroid translations uniform
    in a cube of side 2*half_box around the receptor centroid."""
    u1, u2, u3 = rng.random(n), rng.random(n), rng.random(n)
    a, b = np.sqrt(1.0 - u1), np.sqrt(u1)
    qx, qy = a * np.sin(2 * np.pi * u2), a * np.cos(2 * np.pi * u2)
    qz, qw = b * np.sin(2 * np.pi * u3), b * np.cos(2 * np.pi * u3)
    r00 = 1 - 2 * (qy * qy + qz * qz)
    r10 = 2 * (qx * qy + qz * qw)
    r20 = 2 * (qx * qz - qy * qw)
    r21 = 2 * (qy * qz + qx * qw)
    r22 = 1 - 2 * (qx * qx + qy * qy)
    beta = -np.arcsin(np.clip(r20, -1.0, 1.0))
    alpha = np.arctan2(r10, r00)
    gamma = np.arctan2(r21, r22)
    g = np.empty((n, 6))
    g[:, 0] = np.mod(alpha, 2 * np.pi)
    g[:, 1] = np.mod(beta, 2 * np.pi)
    g[:, 2] = np.mod(gamma, 2 * np.pi)
    g[:, 3:] = rng.uniform(-half_box, half_box, size=(n, 3))
    return g
