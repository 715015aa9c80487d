"""Known-answer tests of the setup layer: the OPLS parameter table and the PDB
reader that pack the inputs of the C ABI.

The table half re-states every assertion of gdock's own tests of its
parameter module (src/toppar.rs:669-880) against ``toppar.json`` through the
same accessors the reader uses (``pdb.atom_type`` = ``get_atom``,
``pdb.type_params(t)[field]`` = ``get_epsilon`` / ``get_rmin2`` /
``get_eps_1_4`` / ``get_rmin2_1_4`` / ``get_charge``; a missing type or field
is ``None``, as the reference's ``Option``).

The reader half pins ``pdb.read_pdb_text`` on hand-written fixed-column
records whose answers follow from the reference's reader
(src/structure.rs:187-300), and re-states the reference's file-level tests
(src/structure.rs:358-362, 522-617) on its data files when a checkout is
named by the environment variable GDOCK_REF.
"""
import os
from pathlib import Path

import numpy as np
import pytest

from gdock_gb300 import pdb


def _param(fn: str, t: str):
    p = pdb.type_params(t)
    if p is None:
        return None
    return p.get(fn)


def get_epsilon(t):
    return _param("epsilon", t)


def get_rmin2(t):
    return _param("rmin2", t)


def get_eps_1_4(t):
    return _param("eps_1_4", t)


def get_rmin2_1_4(t):
    return _param("rmin2_1_4", t)


def get_charge(t):
    return _param("charge", t)


def get_atom(res, name):
    return pdb.atom_type(res, name)


# ---- src/toppar.rs:669-880 -------------------------------------------------

@pytest.mark.parametrize("fn,t,want", [
    (get_epsilon, "C135", -0.066000),       # test_get_epsilon_carbon (:669-674)
    (get_epsilon, "N238", -0.170000),       # test_get_epsilon_nitrogen (:676-681)
    (get_rmin2, "C135", 1.9643086),         # test_get_rmin2_carbon (:689-694)
    (get_rmin2, "H140", 1.4030776),         # test_get_rmin2_hydrogen (:696-701)
    (get_eps_1_4, "C135", -0.033000),       # test_get_eps_1_4_carbon (:709-714)
    (get_eps_1_4, "S200", -0.212500),       # test_get_eps_1_4_sulfur (:716-721)
    (get_rmin2_1_4, "O154", 1.7510408),     # test_get_rmin2_1_4_oxygen (:729-734)
    (get_rmin2_1_4, "CLA", 2.2561487),      # test_get_rmin2_1_4_chloride (:736-741)
])
def test_type_parameters_within_1e6(fn, t, want):
    v = fn(t)
    assert v is not None
    assert abs(v - want) < 1e-6


@pytest.mark.parametrize("fn,t", [
    (get_epsilon, "UNKNOWN"),     # test_get_epsilon_unknown (:683-687)
    (get_rmin2, "INVALID"),       # test_get_rmin2_unknown (:703-707)
    (get_eps_1_4, "NOTFOUND"),    # test_get_eps_1_4_unknown (:723-727)
    (get_rmin2_1_4, "XYZ"),       # test_get_rmin2_1_4_unknown (:743-747)
    (get_charge, "NOTFOUND"),     # test_get_charge_unknown (:827-831)
])
def test_unknown_types_are_none(fn, t):
    assert fn(t) is None


@pytest.mark.parametrize("res,name,want", [
    # test_get_atom_alanine (:749-756)
    ("ALA", "N", "N238"), ("ALA", "CA", "C224"), ("ALA", "CB", "C135"), ("ALA", "C", "C235"), ("ALA", "O", "O236"),
    # test_get_atom_glycine (:758-764)
    ("GLY", "N", "N238"), ("GLY", "CA", "C223"), ("GLY", "C", "C235"), ("GLY", "O", "O236"),
    # test_get_atom_proline (:766-771)
    ("PRO", "N", "N239"), ("PRO", "CD", "C245"), ("PRO", "CA", "C246"),
    # test_get_atom_arginine (:773-779)
    ("ARG", "NE", "N303"), ("ARG", "CZ", "C302"), ("ARG", "NH1", "N300"), ("ARG", "NH2", "N300"),
    # test_get_atom_tryptophan (:781-786)
    ("TRP", "NE1", "N503"), ("TRP", "CG", "C500"), ("TRP", "CD2", "C501"),
    # test_get_atom_histidine_variants (:839-855)
    ("HSD", "ND1", "N503"), ("HSD", "NE2", "N511"), ("HSE", "ND1", "N511"), ("HSE", "NE2", "N503"),
    ("HSP", "ND1", "N512"), ("HSP", "NE2", "N512"), ("HIS", "ND1", "N503"),
])
def test_atom_types(res, name, want):
    assert get_atom(res, name) == want


def test_atom_type_unknowns():
    assert get_atom("XXX", "CA") is None          # test_get_atom_unknown_residue (:788-792)
    assert get_atom("ALA", "NOTEXIST") is None    # test_get_atom_unknown_atom (:794-798)


@pytest.mark.parametrize("t,want", [
    # test_get_charge_backbone (:800-806): exact equality, as assert_eq! on f64
    ("N238", -0.500), ("H241", 0.300), ("C235", 0.500), ("O236", -0.500),
    # test_get_charge_lysine_sidechain (:808-812)
    ("N287", -0.300), ("H290", 0.330),
    # test_get_charge_arginine_sidechain (:814-820)
    ("N303", -0.700), ("H304", 0.440), ("C302", 0.640), ("N300", -0.800),
    # test_get_charge_aspartate (:822-825)
    ("C271", 0.700), ("O272", -0.800),
    # test_get_charge_sulfur (:833-837)
    ("S200", -0.335), ("S202", -0.335),
])
def test_charges_exact(t, want):
    assert get_charge(t) == want


def test_parameters_consistency():  # :857-865
    for fn in (get_epsilon, get_rmin2, get_eps_1_4, get_rmin2_1_4):
        assert fn("C135") is not None


def test_complete_alanine_mapping():  # :867-879
    for name in ("N", "HN", "CA", "HA", "CB", "HB1", "HB2", "HB3", "C", "O"):
        assert get_atom("ALA", name) is not None, name


# ---- the reader (src/structure.rs:187-300) ----------------------------------

def rec(serial, name, resname, chain, resseq, x, y, z, element="", occ="  1.00", tf="  0.00"):
    """One ATOM record laid out column by column (PDB fixed columns: serial
    7-11, name 13-16, resname 18-20, chain 22, resseq 23-26, x/y/z 31-54,
    occupancy 55-60, B-factor 61-66, element 77-78)."""
    line = "ATOM  " + f"{serial:>5}" + " " + f"{name:<4}" + " " + f"{resname:>3}" + " " + chain
    line += f"{resseq:>4}" + " " + "   " + f"{x:>8.3f}{y:>8.3f}{z:>8.3f}"
    if occ is None:
        return line
    line += occ + tf
    if element:
        line += " " * 10 + f"{element:>2}"
    return line


def test_single_model_without_model_records():
    text = "\n".join([rec(1, "N", "ALA", "A", 1, 0, 0, 0, "N"), rec(2, "CA", "ALA", "A", 1, 1.5, 0, 0, "C"),
                      "TER", "END"])
    models = pdb.read_pdb_text(text)
    assert len(models) == 1 and len(models[0]) == 2
    assert list(models[0].serial) == [1, 2]
    assert models[0].x[1] == 1.5


def test_model_records_give_one_molecule_each():
    body = [rec(1, "N", "GLY", "B", 5, 0, 0, 0, "N"), rec(2, "CA", "GLY", "B", 5, 1, 2, 3, "C")]
    text = "\n".join(["MODEL        1", *body, "ENDMDL", "MODEL        2", *body, "ENDMDL",
                      "MODEL        3", *body, "ENDMDL"])
    models = pdb.read_pdb_text(text)
    assert len(models) == 3
    assert all(len(m) == 2 for m in models)


def test_model_without_endmdl_is_dropped():
    # with MODEL records present, only ENDMDL pushes a molecule (:281-297)
    body = [rec(1, "N", "GLY", "B", 5, 0, 0, 0, "N")]
    text = "\n".join(["MODEL        1", *body, "ENDMDL", "MODEL        2", *body])
    assert len(pdb.read_pdb_text(text)) == 1


def test_short_and_non_atom_lines_are_skipped():
    good = rec(1, "CA", "ALA", "A", 1, 1, 2, 3, "C")
    short = good[:53]                                          # < 54 bytes (:188-190)
    het = "HETATM" + good[6:]                                  # only "ATOM" records
    bad_serial = good[:6] + "  x1 " + good[11:]                # serial must parse (:206)
    bad_resseq = good[:22] + "  ?1" + good[26:]                # resseq must parse (:221)
    bad_x = good[:30] + "   abc  " + good[38:]                 # coordinates must parse (:227-233)
    models = pdb.read_pdb_text("\n".join([short, het, bad_serial, bad_resseq, bad_x, good]))
    assert len(models) == 1 and len(models[0]) == 1


def test_optional_columns_and_element_fallback():
    # no occupancy / B-factor / element columns: 1.0, 0.0 and the first
    # character of the atom name (:235-247)
    line = rec(7, "OG1", "THR", "A", 3, 1, 1, 1, occ=None)
    assert len(line) == 54
    m = pdb.read_pdb_text(line)[0]
    assert m.occupancy[0] == 1.0 and m.tempfactor[0] == 0.0
    assert m.element == ["O"]
    assert m.vdw_radius[0] == 1.52


@pytest.mark.parametrize("element,radius", [
    ("H", 1.2), ("C", 1.7), ("N", 1.55), ("O", 1.52),
    ("S", 1.0),    # sulfur falls to the default: SULFUR_RADIUS is never used (:250-256)
    ("FE", 1.0),
])
def test_vdw_radius_by_element(element, radius):
    m = pdb.read_pdb_text(rec(1, "X1", "ALA", "A", 1, 0, 0, 0, element))[0]
    assert m.vdw_radius[0] == radius


def test_parameters_from_the_table():
    # ALA CB -> C135; an unknown residue or atom name keeps zeros (:258-267)
    text = "\n".join([rec(1, "CB", "ALA", "A", 1, 0, 0, 0, "C"), rec(2, "CB", "XXX", "A", 2, 0, 0, 0, "C"),
                      rec(3, "QQ", "ALA", "A", 3, 0, 0, 0, "C")])
    m = pdb.read_pdb_text(text)[0]
    p = pdb.type_params("C135")
    assert (m.epsilon[0], m.rmin2[0], m.eps_1_4[0], m.rmin2_1_4[0], m.charge[0]) == (
        p["epsilon"], p["rmin2"], p["eps_1_4"], p["rmin2_1_4"], p["charge"])
    for i in (1, 2):
        assert (m.epsilon[i], m.rmin2[i], m.eps_1_4[i], m.rmin2_1_4[i], m.charge[i]) == (0.0,) * 5


# ---- the reference's file-level tests, on its own data ----------------------

def _ref_data():
    root = os.environ.get("GDOCK_REF")
    if not root:
        pytest.skip("GDOCK_REF (a gdock checkout) not set")
    d = Path(root) / "data"
    if not d.is_dir():
        pytest.skip(f"no data directory under GDOCK_REF={root}")
    return d


def test_read_pdb_reference_complex():  # src/structure.rs:358-362 and 598-616
    models = pdb.read_pdb(_ref_data() / "2oob.pdb")
    assert len(models) == 1 and len(models[0]) > 0


def test_read_pdb_single_model_file():  # src/structure.rs:539-558
    models = pdb.read_pdb(_ref_data() / "1h590A_0A.pdb")
    assert len(models) == 1 and len(models[0]) > 0


def test_read_pdb_multi_model_file():  # src/structure.rs:560-596
    models = pdb.read_pdb(_ref_data() / "1h590B_0A_poses.pdb")
    assert len(models) > 1
    n0 = len(models[0])
    assert n0 > 0 and all(len(m) == n0 for m in models)
    # the same structure in every MODEL: names and residues agree model by model
    assert all(m.name == models[0].name and np.array_equal(m.resseq, models[0].resseq) for m in models)


def test_toppar_json_is_the_reference_table():
    """The shipped table equals a fresh extraction from the reference's
    src/toppar.rs (both parameter tables and the residue -> atom-type map)."""
    import importlib.util
    import json
    src = Path(os.environ.get("GDOCK_REF", "")) / "src" / "toppar.rs"
    _ref_data()
    if not src.exists():
        pytest.skip(f"no src/toppar.rs under GDOCK_REF={os.environ['GDOCK_REF']}")
    here = Path(pdb.__file__).parent / "data"
    spec = importlib.util.spec_from_file_location("make_toppar", here / "make_toppar.py")
    mk = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mk)
    assert mk.extract(str(src)) == json.loads((here / "toppar.json").read_text())
