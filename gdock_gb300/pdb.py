"""PDB reading/writing and per-atom parameter assignment (host-side setup).

This is the input-packing layer that sits in front of the GPU path: it turns
PDB text into the structure-of-arrays form the C ABI takes.  It follows
gdock's reader field by field:

* fixed-column ATOM parsing, lines shorter than 54 bytes or not starting with
  ``ATOM`` ignored, serial/resseq/x/y/z required (src/structure.rs:187-233);
* occupancy/B-factor optional (src/structure.rs:235-239);
* element from columns 77-78, else the first character of the atom name
  (src/structure.rs:241-247);
* van der Waals radius by element, H 1.2 / C 1.7 / N 1.55 / O 1.52 and 1.0
  for everything else, sulfur included (src/structure.rs:249-256,
  src/constants.rs:68-72);
* epsilon, Rmin/2, their 1-4 variants and charge through the residue/atom
  name -> atom type table (src/structure.rs:258-267, src/toppar.rs);
* MODEL/ENDMDL handling, including dropping a trailing model that has no
  ENDMDL (src/structure.rs:273-300).
"""
from __future__ import annotations

import json
from dataclasses import dataclass, field
from pathlib import Path
from typing import List

import numpy as np

_TOPPAR = json.loads((Path(__file__).parent / "data" / "toppar.json").read_text())

# element classes used by the C ABI (gd_atoms.element)
ELEM_OTHER, ELEM_H, ELEM_C, ELEM_N, ELEM_O, ELEM_S = 0, 1, 2, 3, 4, 5
_ELEM_CLASS = {"H": ELEM_H, "C": ELEM_C, "N": ELEM_N, "O": ELEM_O, "S": ELEM_S}
# src/structure.rs:250-256 (radius by trimmed element; S falls to 1.0)
_VDW_RADIUS = {"H": 1.2, "C": 1.7, "N": 1.55, "O": 1.52}


def atom_type(resname: str, name: str):
    """Residue name + atom name -> OPLS atom type (src/toppar.rs:152-581)."""
    res = _TOPPAR["residues"].get(resname)
    if res is None:
        return None
    return res.get(name)


def type_params(t: str):
    return _TOPPAR["types"].get(t)


def residue_atom_names(resname: str) -> List[str]:
    return list(_TOPPAR["residues"][resname].keys())


@dataclass
class Molecule:
    """Atoms of one molecule as parallel arrays (one entry per ATOM record)."""
    serial: np.ndarray
    name: List[str]
    altloc: List[str]
    resname: List[str]
    chainid: List[str]
    resseq: np.ndarray
    icode: List[str]
    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    occupancy: np.ndarray
    tempfactor: np.ndarray
    element: List[str]
    charge: np.ndarray
    vdw_radius: np.ndarray
    epsilon: np.ndarray
    rmin2: np.ndarray
    eps_1_4: np.ndarray
    rmin2_1_4: np.ndarray

    def __len__(self) -> int:
        return int(self.x.shape[0])

    # -- derived arrays consumed by the C ABI --------------------------------
    @property
    def element_class(self) -> np.ndarray:
        return np.array([_ELEM_CLASS.get(e.strip(), ELEM_OTHER) for e in self.element], dtype=np.uint8)

    @property
    def chain_code(self) -> np.ndarray:
        return np.array([ord(c) if c else 32 for c in self.chainid], dtype=np.uint8)

    @property
    def is_ca(self) -> np.ndarray:
        return np.array([n.strip() == "CA" for n in self.name], dtype=np.uint8)

    def xyz(self) -> np.ndarray:
        return np.stack([self.x, self.y, self.z], axis=1)

    def with_coords(self, x, y, z) -> "Molecule":
        d = dict(self.__dict__)
        d["x"] = np.ascontiguousarray(x, dtype=np.float64)
        d["y"] = np.ascontiguousarray(y, dtype=np.float64)
        d["z"] = np.ascontiguousarray(z, dtype=np.float64)
        return Molecule(**d)

    def center_of_mass(self):
        """Unweighted centroid, summed left to right (src/structure.rs:63-69)."""
        n = float(len(self))
        sx = sy = sz = -0.0
        for v in self.x.tolist():
            sx += v
        for v in self.y.tolist():
            sy += v
        for v in self.z.tolist():
            sz += v
        return (sx / n, sy / n, sz / n)


def _build(rows) -> Molecule:
    cols = list(zip(*rows)) if rows else [[] for _ in range(19)]
    f64 = lambda c: np.array(c, dtype=np.float64)
    return Molecule(
        serial=np.array(cols[0], dtype=np.int32), name=list(cols[1]), altloc=list(cols[2]),
        resname=list(cols[3]), chainid=list(cols[4]), resseq=np.array(cols[5], dtype=np.int16),
        icode=list(cols[6]), x=f64(cols[7]), y=f64(cols[8]), z=f64(cols[9]),
        occupancy=np.array(cols[10], dtype=np.float32), tempfactor=np.array(cols[11], dtype=np.float32),
        element=list(cols[12]), charge=f64(cols[13]), vdw_radius=f64(cols[14]), epsilon=f64(cols[15]),
        rmin2=f64(cols[16]), eps_1_4=f64(cols[17]), rmin2_1_4=f64(cols[18]))


def _parse_int(s: str, lo: int, hi: int):
    s = s.strip()
    if not s or not (s.lstrip("+-").isdigit()):
        return None
    v = int(s)
    return v if lo <= v <= hi else None


def _parse_float(s: str):
    s = s.strip()
    try:
        if "_" in s:
            return None
        return float(s)
    except ValueError:
        return None


def process_atom_line(line: str):
    """One ATOM record -> tuple of fields, or None (src/structure.rs:187-270)."""
    if not line.startswith("ATOM") or len(line) < 54:
        return None

    def get(a, b):
        return line[a:b] if len(line) >= b else ""

    serial = _parse_int(get(6, 11), -2**31, 2**31 - 1)
    if serial is None:
        return None
    name = get(12, 16).strip()
    altloc = get(16, 17)[:1] or " "
    resname = get(17, 20).strip()
    chainid = get(21, 22)[:1] or " "
    resseq = _parse_int(get(22, 26), -32768, 32767)
    if resseq is None:
        return None
    icode = get(26, 27)[:1] or " "
    x, y, z = _parse_float(get(30, 38)), _parse_float(get(38, 46)), _parse_float(get(46, 54))
    if x is None or y is None or z is None:
        return None
    occ = _parse_float(get(54, 60))
    occ = 1.0 if occ is None else occ
    tf = _parse_float(get(60, 66))
    tf = 0.0 if tf is None else tf
    element = get(76, 78).strip()
    if not element:
        element = name[:1] if name else " "
    vdw = _VDW_RADIUS.get(element.strip(), 1.0)
    eps = rmin2 = eps14 = rmin14 = charge = 0.0
    t = atom_type(resname, name)
    if t is not None:
        p = type_params(t) or {}
        eps = p.get("epsilon", 0.0)
        rmin2 = p.get("rmin2", 0.0)
        eps14 = p.get("eps_1_4", 0.0)
        rmin14 = p.get("rmin2_1_4", 0.0)
        charge = p.get("charge", 0.0)
    return (serial, name, altloc, resname, chainid, resseq, icode, x, y, z, occ, tf,
            element, charge, vdw, eps, rmin2, eps14, rmin14)


def read_pdb_text(text: str) -> List[Molecule]:
    """All models of a PDB text (src/structure.rs:273-300)."""
    models: List[Molecule] = []
    rows = []
    has_model = False
    for line in text.splitlines():
        if line.startswith("MODEL"):
            has_model = True
            rows = []
        elif line.startswith("ENDMDL"):
            models.append(_build(rows))
            rows = []
        else:
            a = process_atom_line(line)
            if a is not None:
                rows.append(a)
    if not has_model:
        models.append(_build(rows))
    return models


def read_pdb(path) -> List[Molecule]:
    return read_pdb_text(Path(path).read_text())


def atom_line(serial, name, resname, chainid, resseq, x, y, z, element, occ=1.0, tf=0.0) -> str:
    """One fixed-column ATOM record in the layout gdock writes (src/structure.rs:159-176)."""
    nm = name if len(name) >= 4 else f"{name:^4}"
    return (f"ATOM  {serial:>5} {nm:<4} {resname:<3} {chainid:>1}{resseq:>4}    "
            f"{x:>8.3f}{y:>8.3f}{z:>8.3f}{occ:>6.2f}{tf:>6.2f}          {element:>2}\n")


def write_pdb_text(mol: Molecule) -> str:
    out = []
    for i in range(len(mol)):
        out.append(atom_line(int(mol.serial[i]), mol.name[i], mol.resname[i], mol.chainid[i],
                             int(mol.resseq[i]), mol.x[i], mol.y[i], mol.z[i], mol.element[i],
                             float(mol.occupancy[i]), float(mol.tempfactor[i])))
    return "".join(out)


def combine_molecules(receptor: Molecule, ligand: Molecule) -> Molecule:
    """Receptor atoms then ligand atoms (src/commands/run.rs:35-49)."""
    d = {}
    for k, v in receptor.__dict__.items():
        w = ligand.__dict__[k]
        d[k] = np.concatenate([v, w]) if isinstance(v, np.ndarray) else list(v) + list(w)
    return Molecule(**d)


def position_ligand(receptor: Molecule, ligand: Molecule) -> Molecule:
    """Move the ligand centroid onto the receptor centroid (src/utils.rs:77-95):
    x <- (x - lx) + rx, each centroid summed left to right."""
    rx, ry, rz = receptor.center_of_mass()
    lx, ly, lz = ligand.center_of_mass()
    return ligand.with_coords((ligand.x - lx) + rx, (ligand.y - ly) + ry, (ligand.z - lz) + rz)


def restraint_pairs_to_indices(receptor: Molecule, ligand: Molecule, pairs):
    """Resolve (receptor resseq, ligand resseq) pairs to CA atom indices: the
    first atom named CA with that residue number in each molecule; pairs with
    a missing CA are dropped (src/restraints.rs:44-77)."""
    def first_ca(mol, res):
        for i in range(len(mol)):
            if mol.name[i].strip() == "CA" and int(mol.resseq[i]) == int(res):
                return i
        return -1
    out = []
    for r, l in pairs:
        a, b = first_ca(receptor, r), first_ca(ligand, l)
        if a >= 0 and b >= 0:
            out.append((a, b))
    return out
