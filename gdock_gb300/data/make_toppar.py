"""Regenerate ``toppar.json`` from gdock's parameter module.

gdock assigns per-atom force-field parameters at PDB parse time from an
OPLS-AA table (``src/toppar.rs``): residue name + atom name -> atom type
(``get_atom``, src/toppar.rs:152-581), and atom type -> epsilon, Rmin/2,
their 1-4 variants and partial charge (src/toppar.rs:12-129, 583-663).
The values are data that must be identical for parity, so this script reads
them out of the reference's source once and writes them as JSON; the JSON
is what the package ships.

Usage: python gdock_gb300/data/make_toppar.py [path/to/gdock/src/toppar.rs]
(default: $GDOCK_REF/src/toppar.rs, GDOCK_REF naming a gdock checkout)
"""
import json
import os
import re
import sys
from pathlib import Path


def _fn_body(src: str, name: str) -> str:
    start = src.index(f"pub fn {name}(")
    # the body ends at the first line that is exactly "}" after start
    end = src.index("\n}\n", start)
    return src[start:end]


def _type_table(src: str, name: str) -> dict:
    """Parse `match atom { "A" | "B" => Some(v), ... }` into {type: v}."""
    body = _fn_body(src, name)
    out = {}
    for m in re.finditer(r'((?:"[A-Z0-9]+"\s*\|?\s*)+)=>\s*\{?\s*Some\(\s*(-?[0-9.]+)\s*\)', body):
        keys = re.findall(r'"([A-Z0-9]+)"', m.group(1))
        for k in keys:
            out[k] = m.group(2)  # keep the literal text; parsed as float later
    return out


def _residue_table(src: str) -> dict:
    body = _fn_body(src, "get_atom")
    out = {}
    for m in re.finditer(r'((?:"[A-Z0-9]+"\s*\|?\s*)+)=>\s*match atom_name \{(.*?)\n        \},', body, re.S):
        resnames = re.findall(r'"([A-Z0-9]+)"', m.group(1))
        atoms = dict(re.findall(r'"([A-Z0-9\']+)"\s*=>\s*Some\("([A-Z0-9]+)"\)', m.group(2)))
        for r in resnames:
            out[r] = atoms
    return out


def extract(path: str) -> dict:
    """The parameter and residue tables of ``toppar.rs`` as the JSON document."""
    src = Path(path).read_text()
    tables = {k: _type_table(src, k) for k in
              ("get_epsilon", "get_rmin2", "get_eps_1_4", "get_rmin2_1_4", "get_charge")}
    types = {}
    for fn, tab in tables.items():
        for t, v in tab.items():
            types.setdefault(t, {})[fn[4:]] = float(v)
    doc = {
        "source": "gdock src/toppar.rs (OPLS-AA/M values)",
        "types": dict(sorted(types.items())),
        "residues": _residue_table(src),
    }
    return doc


def main(path: str) -> None:
    doc = extract(path)
    out = Path(__file__).with_name("toppar.json")
    out.write_text(json.dumps(doc, indent=1, sort_keys=True) + "\n")
    print(f"wrote {out}: {len(doc['types'])} types, {len(doc['residues'])} residues")


if __name__ == "__main__":
    if len(sys.argv) > 1:
        main(sys.argv[1])
    elif os.environ.get("GDOCK_REF"):
        main(str(Path(os.environ["GDOCK_REF"]) / "src" / "toppar.rs"))
    else:
        sys.exit("usage: make_toppar.py path/to/src/toppar.rs (or set GDOCK_REF to a gdock checkout)")
