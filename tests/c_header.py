"""A small reader of the library's C headers (include/*.h): structs (fields
in order, with array lengths), opaque handles, enums, numeric #defines and
function prototypes.  The headers use one plain C subset (no function
pointers, no nested declarations), which is all this reader accepts; it is
test infrastructure for checking bindings written in other languages."""
from __future__ import annotations

import re
from pathlib import Path

HEADERS = ["voidray_gpu.h", "voidray_denoise.h", "voidray_assets.h"]


def _strip(text: str) -> str:
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    return re.sub(r"//[^\n]*", " ", text)


def _ctype(tok: str) -> tuple[str, int, tuple]:
    """'const float * const *' -> (base, pointer depth, per pointer level from
    the innermost: whether what it points to is const)."""
    t = tok.replace("*", " * ").split()
    stars = [i for i, x in enumerate(t) if x == "*"]
    consts = tuple("const" in t[(stars[k - 1] + 1 if k else 0):stars[k]] for k in range(len(stars)))
    base = " ".join(x for x in t if x not in ("*", "const", "struct", "enum"))
    return base, len(stars), consts


def _decl(d: str):
    """'const float* positions' / 'float org[3]' -> (name, (base, depth, const), array length or 0)."""
    d = d.strip()
    m = re.match(r"^(.*?)([A-Za-z_]\w*)\s*(?:\[(\w+)\])?$", d)
    if not m:
        raise ValueError(f"cannot read declaration {d!r}")
    ty, name, arr = m.groups()
    return name, _ctype(ty), int(arr) if arr and arr.isdigit() else (arr or 0)


def read(include_dir: Path) -> dict:
    out = {"structs": {}, "opaque": set(), "enums": {}, "defines": {}, "functions": {}}
    for h in HEADERS:
        text = _strip((include_dir / h).read_text())
        for m in re.finditer(r"#define\s+(VR_\w+)\s+\(?(0x[0-9A-Fa-f]+|\d+)u?(?:\s*<<\s*(\d+))?\)?", text):
            v = int(m.group(2), 0) << int(m.group(3) or 0)
            out["defines"][m.group(1)] = v
        body = re.sub(r"#[^\n]*", " ", text)
        for m in re.finditer(r"typedef\s+struct\s+(\w+)\s*\{(.*?)\}\s*(\w+)\s*;", body, flags=re.S):
            fields = []
            for stmt in m.group(2).split(";"):
                stmt = stmt.strip()
                if not stmt:
                    continue
                first, *rest = [x.strip() for x in stmt.split(",")]
                name, ty, arr = _decl(first)
                fields.append((name, ty, arr))
                base = first[: first.rindex(name)].replace("*", "").strip()
                for extra in rest:
                    fields.append(_decl(base + " " + extra))
            out["structs"][m.group(3)] = fields
        for m in re.finditer(r"typedef\s+struct\s+(\w+)\s+(\w+)\s*;", body):
            out["opaque"].add(m.group(2))
        for m in re.finditer(r"(?:typedef\s+)?enum\s*(\w*)\s*\{(.*?)\}\s*(\w*)\s*;", body, flags=re.S):
            vals = {}
            for item in m.group(2).split(","):
                if "=" in item:
                    k, v = item.split("=")
                    vals[k.strip()] = int(v.strip(), 0)
            out["enums"][m.group(3) or m.group(1) or f"anon{len(out['enums'])}"] = vals
        body = re.sub(r"typedef\s+(struct|enum)\s*\w*\s*\{.*?\}\s*\w*\s*;", " ", body, flags=re.S)
        body = re.sub(r"typedef\s+struct\s+\w+\s+\w+\s*;", " ", body)
        body = re.sub(r"enum\s*\{.*?\}\s*;", " ", body, flags=re.S)
        body = body.replace('extern "C" {', " ").replace("}", " ")
        for m in re.finditer(r"([\w\s\*]+?)\b(vr_\w+)\s*\(([^)]*)\)\s*;", body):
            ret = _ctype(m.group(1).strip())
            params = []
            p = m.group(3).strip()
            if p and p != "void":
                for d in p.split(","):
                    name, ty, _ = _decl(d)
                    params.append((name, ty))
            out["functions"][m.group(2)] = (ret, params)
    return out
