"""The Rust FFI crate (gdock-gb300-sys/src/lib.rs) against the C header
(include/gdock_gb300.h): every entry point with the same name, argument count
and argument types in order and the same return type; every struct with the
same fields, in order, of the same types; every constant with the same value.

Cargo is not available in this image, so the crate is not compiled here: this
check is textual, on both files' declarations."""
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "gdock_gb300.h"
CRATE = ROOT / "gdock-gb300-sys" / "src" / "lib.rs"

SCALARS = {"int32_t": "i32", "uint32_t": "u32", "int64_t": "i64", "uint64_t": "u64", "int16_t": "i16",
           "uint8_t": "u8", "double": "f64", "char": "c_char", "void": "c_void", "gd_status": "gd_status",
           "gd_precision": "gd_precision"}


def _strip_c_comments(s):
    return re.sub(r"/\*.*?\*/", "", s, flags=re.S)


def c_type_to_rust(decl: str):
    """'const gd_pose_frame *d_frames' -> ('d_frames', '*const gd_pose_frame')."""
    decl = " ".join(decl.replace("*", " * ").split())
    toks = decl.split(" ")
    name = toks[-1]
    arr = re.match(r"(\w+)\[(\d+)\]$", name)
    if arr:
        name = arr.group(1)
    toks = toks[:-1]
    # const flags: c[0] for the base type, c[i] for the i-th pointer
    consts, base = [False], None
    for t in toks:
        if t == "const":
            consts[-1] = True
        elif t == "*":
            consts.append(False)
        else:
            base = t
    rust = SCALARS.get(base, base)
    for c in consts[:-1]:
        rust = f"*{'const' if c else 'mut'} {rust}"
    if arr:
        rust = f"[{rust}; {arr.group(2)}]"
    return name, rust


def header_functions():
    h = _strip_c_comments(HEADER.read_text())
    out = {}
    for m in re.finditer(r"^([A-Za-z_][\w \*]*?)\b(gd_\w+)\s*\(([^)]*)\)\s*;", h, flags=re.M):
        ret = c_type_to_rust(m.group(1).strip() + " r")[1]
        args = [] if m.group(3).strip() == "void" else [c_type_to_rust(a) for a in m.group(3).split(",")]
        out[m.group(2)] = (args, ret)
    return out


def header_structs():
    h = _strip_c_comments(HEADER.read_text())
    out = {}
    for m in re.finditer(r"typedef struct (\w+)\s*\{(.*?)\}\s*\w+;", h, flags=re.S):
        fields = []
        for stmt in m.group(2).split(";"):
            stmt = " ".join(stmt.split())
            if not stmt:
                continue
            parts = [p.strip() for p in stmt.split(",")]
            first = c_type_to_rust(parts[0])
            fields.append(first)
            # 'const double *x, *y, *z' and 'double vdw, elec': the base type
            # of the first declarator, each later one with its own stars
            base = parts[0][: parts[0].rfind(first[0])].replace("*", "").strip()
            for p in parts[1:]:
                fields.append(c_type_to_rust(base + " " + p))
        out[m.group(1)] = fields
    return out


def header_constants():
    h = _strip_c_comments(HEADER.read_text())
    out = {}
    for m in re.finditer(r"\b(GD_[A-Z0-9_]+)\s*=\s*(\d+)", h):
        out[m.group(1)] = int(m.group(2))
    for m in re.finditer(r"#define\s+(GD_[A-Z0-9_]+)\s+(\d+)", h):
        out[m.group(1)] = int(m.group(2))
    return out


def _split_top(s):
    parts, depth, cur = [], 0, ""
    for ch in s:
        if ch == "[":
            depth += 1
        elif ch == "]":
            depth -= 1
        if ch == "," and depth == 0:
            parts.append(cur)
            cur = ""
        else:
            cur += ch
    if cur.strip():
        parts.append(cur)
    return [p.strip() for p in parts if p.strip()]


def crate_text():
    return re.sub(r"//[^\n]*", "", CRATE.read_text())


def crate_functions():
    src = crate_text()
    block = src[src.index('extern "C" {'):]
    block = block[: block.index("\n}\n")]
    out = {}
    for m in re.finditer(r"pub fn (\w+)\((.*?)\)\s*(?:->\s*([^;]+))?;", block, flags=re.S):
        args = []
        for a in _split_top(m.group(2)):
            n, t = a.split(":", 1)
            args.append((n.strip(), " ".join(t.split())))
        out[m.group(1)] = (args, " ".join((m.group(3) or "()").split()))
    return out


def crate_structs():
    src = crate_text()
    out = {}
    for m in re.finditer(r"#\[repr\(C\)\][^\n]*\n(?:#\[[^\n]*\]\n)*pub struct (\w+) \{(.*?)\n\}", src, flags=re.S):
        fields = []
        for f in re.finditer(r"pub (\w+): ([^\n]+?),?\n", m.group(2) + "\n"):
            fields.append((f.group(1), " ".join(f.group(2).rstrip(",").split())))
        if fields:
            out[m.group(1)] = fields
    return out


def crate_constants():
    out = {}
    for m in re.finditer(r"pub const (GD_[A-Z0-9_]+): \w+ = (\d+);", crate_text()):
        out[m.group(1)] = int(m.group(2))
    return out


def test_every_entry_point_matches():
    h, r = header_functions(), crate_functions()
    assert len(h) > 40
    assert sorted(h) == sorted(r), (set(h) ^ set(r))
    for name, (args, ret) in h.items():
        rargs, rret = r[name]
        assert [t for _, t in rargs] == [t for _, t in args], name
        assert [n for n, _ in rargs] == [n for n, _ in args], name
        assert rret == ret, (name, rret, ret)


def test_every_struct_matches():
    h, r = header_structs(), crate_structs()
    assert sorted(h) == sorted(r), (set(h) ^ set(r))
    for name, fields in h.items():
        assert r[name] == fields, name


def test_every_constant_matches():
    h, r = header_constants(), crate_constants()
    missing = set(h) - set(r)
    assert not missing, missing
    for k, v in h.items():
        assert r[k] == v, k


def test_no_placeholders_in_the_crate():
    src = crate_text()
    for word in ("todo!", "unimplemented!", "..todo"):
        assert word not in src


@pytest.mark.parametrize("patch", sorted((ROOT / "integration").glob("*.patch")), ids=lambda p: p.name)
def test_integration_patches_are_unified_diffs(patch):
    """Each patch names its gdock file and holds well-formed hunks whose
    line counts agree with their headers."""
    text = patch.read_text()
    files = re.findall(r"^\+\+\+ b/(\S+)", text, flags=re.M)
    assert files, patch.name
    for hunk in re.finditer(r"^@@ -(\d+)(?:,(\d+))? \+(\d+)(?:,(\d+))? @@[^\n]*\n((?:[ +\-\\][^\n]*\n?)*)", text,
                            flags=re.M):
        old_n = int(hunk.group(2) or 1)
        new_n = int(hunk.group(4) or 1)
        lines = [l for l in hunk.group(5).split("\n") if l and not l.startswith("\\")]
        lines = lines[: sum(1 for _ in lines)]
        o = sum(1 for l in lines if l[0] in " -")
        n = sum(1 for l in lines if l[0] in " +")
        assert (o, n) == (old_n, new_n), (patch.name, hunk.group(0)[:80])


def test_integration_patches_apply_to_gdock(tmp_path):
    """With a gdock checkout named by GDOCK_REF, the patches apply to a copy
    of its sources in order, each without fuzz or offset complaints."""
    import os
    import shutil
    import subprocess
    ref = os.environ.get("GDOCK_REF")
    if not ref or not (Path(ref) / "src").is_dir():
        pytest.skip("GDOCK_REF (a gdock checkout) not set")
    if shutil.which("patch") is None:
        pytest.skip("no patch tool")
    work = tmp_path / "gdock"
    shutil.copytree(Path(ref) / "src", work / "src")
    shutil.copy(Path(ref) / "Cargo.toml", work / "Cargo.toml")
    for p in sorted((ROOT / "integration").glob("*.patch")):
        r = subprocess.run(["patch", "-p1", "--no-backup-if-mismatch", "-i", str(p)], cwd=work,
                           capture_output=True, text=True)
        assert r.returncode == 0, (p.name, r.stdout, r.stderr)
        assert "fuzz" not in r.stdout and "offset" not in r.stdout, (p.name, r.stdout)
    assert (work / "src" / "gpu.rs").exists()
