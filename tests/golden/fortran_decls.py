"""A small reader of Fortran 90 procedure interfaces: procedure headers, dummy-argument order and the declared
type, kind and rank of each dummy.  Used by tests/golden/make_interfaces.py (to record the reference's interfaces)
and by tests/test_fortran_layer.py (to read the replacement modules of wtb_gb300/fortran the same way)."""
from __future__ import annotations

import re

_HDR = re.compile(r"^\s*(?:(?:recursive|pure|elemental)\s+)*(?:(complex\(8\)|real\(8\)|double\s+precision|double\s+complex|"
                  r"integer|logical)\s+)?(subroutine|function)\s+(\w+)\s*\(([^)]*)\)", re.I)
_END = re.compile(r"^\s*end\s+(subroutine|function)\b", re.I)
_DECL = re.compile(r"^\s*(integer|real|double\s+precision|double\s+complex|complex|character|logical|type)\b(.*?)::(.*)$",
                   re.I)


def _strip_comment(line: str) -> str:
    out, q = [], None
    for ch in line:
        if q:
            out.append(ch)
            if ch == q:
                q = None
        elif ch in "'\"":
            q = ch
            out.append(ch)
        elif ch == "!":
            break
        else:
            out.append(ch)
    return "".join(out)


def logical_lines(text: str) -> list[str]:
    """Comment-free statements with continuation lines joined."""
    out, cur = [], ""
    for raw in text.splitlines():
        s = _strip_comment(raw).rstrip()
        if cur:
            s = s.lstrip()
            if s.startswith("&"):
                s = s[1:]
        if s.endswith("&"):
            cur += s[:-1]
            continue
        out.append(cur + s)
        cur = ""
    if cur:
        out.append(cur)
    return out


def _norm_type(base: str, attrs: str) -> tuple[str, str | None]:
    b = re.sub(r"\s+", "", base.lower())
    a = re.sub(r"\s+", "", attrs.lower())
    if b in ("doubleprecision",) or (b == "real" and a.startswith("(8)")) or (b == "real" and a.startswith("(kind=8)")):
        t = "real8"
    elif b == "real":
        t = "real4"
    elif b in ("doublecomplex",) or (b == "complex" and (a.startswith("(8)") or a.startswith("(kind=8)"))):
        t = "complex8"
    elif b == "integer":
        t = "integer"
    elif b == "logical":
        t = "logical"
    elif b == "character":
        m = re.match(r"\(len=(\d+|\*)\)", a)
        t = "character" + (m.group(1) if m else "1")
    else:
        t = b + a.split(",")[0]
    dims = None
    m = re.search(r"dimension\(([^)]*)\)", a)
    if m:
        dims = m.group(1)
    return t, dims


def _split_names(s: str) -> list[tuple[str, str | None]]:
    out, depth, cur = [], 0, ""
    for ch in s:
        if ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        if ch == "," and depth == 0:
            out.append(cur)
            cur = ""
        else:
            cur += ch
    out.append(cur)
    res = []
    for item in out:
        item = item.strip()
        if not item:
            continue
        item = item.split("=")[0].strip()
        m = re.match(r"(\w+)\s*(?:\((.*)\))?", item)
        if m:
            res.append((m.group(1).lower(), m.group(2)))
    return res


def _rank(dims: str | None) -> int:
    if dims is None:
        return 0
    depth, n = 0, 1
    for ch in dims:
        if ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        elif ch == "," and depth == 0:
            n += 1
    return n


def procedures(text: str) -> dict:
    """{name: {"kind": subroutine|function, "result": type or None, "args": [names], "types": {arg: [type, rank,
    assumed_shape]}}} for every procedure in the text (nested procedures included)."""
    lines = logical_lines(text)
    procs, stack = {}, []
    for ln in lines:
        m = _HDR.match(ln)
        if m and not re.match(r"^\s*end\b", ln, re.I):
            name = m.group(3).lower()
            args = [a.strip().lower() for a in m.group(4).split(",") if a.strip()]
            res = m.group(1)
            rb = res.split("(")[0] if res else None
            procs[name] = {"kind": m.group(2).lower(), "result": _norm_type(rb, res[len(rb):])[0] if res else None,
                           "args": args, "types": {}}
            stack.append(name)
            continue
        if _END.match(ln):
            if stack:
                stack.pop()
            continue
        if not stack:
            continue
        d = _DECL.match(ln)
        if not d:
            continue
        cur = procs[stack[-1]]
        t, dims = _norm_type(d.group(1), d.group(2))
        for nm, ndims in _split_names(d.group(3)):
            if nm in cur["args"] and nm not in cur["types"]:
                dd = ndims if ndims is not None else dims
                cur["types"][nm] = [t, _rank(dd), bool(dd) and set(dd.replace(",", "").strip()) == {":"}]
            if cur["kind"] == "function" and nm == stack[-1] and cur["result"] is None:
                cur["result"] = t
    return procs
