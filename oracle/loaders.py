"""Mesh decoders restated in Python (TEST INFRASTRUCTURE ONLY): the checker for the library's
`.tri` / `.obj` decoders.

`.tri` follows the reference's lexer (bvhtracer/tri_loader/src/lexer.rs: whitespace ' ', '\\t',
'\\\\'; '\\n' and '\\r' are tokens; '#' at a token's start skips the line) and loader
(tri_loader/src/loader.rs:94-186: triangles of nine floats, "\\n" tokens between triangles,
ExpectedFloat / EndOfFile with the line number), and TriMeshDecoder's face normal
(bvhtracer/src/mesh/decoders.rs:120-129).  Floats are converted with exact rational arithmetic
and round-half-to-even to binary32 (the correctly rounded result Rust's `str::parse::<f32>`
gives), not with a C library call, so the check is independent of the library's strtof.
"""
from __future__ import annotations

import re
from fractions import Fraction

import numpy as np

_RUST_FLOAT = re.compile(r"^[+-]?(?:\d+\.?\d*|\.\d+)(?:[eE][+-]?\d+)?$")
_SPECIAL = {"inf", "infinity", "nan"}


class DecodeError(ValueError):
    def __init__(self, line, kind, token=""):
        super().__init__(f"line {line}: {kind} {token!r}")
        self.line, self.kind, self.token = line, kind, token


def _round_f32(x: Fraction) -> np.float32:
    """Binary32 nearest to the rational x, ties to even (overflow to inf, subnormals kept)."""
    if x == 0:
        return np.float32(0.0)
    sign = -1.0 if x < 0 else 1.0
    x = abs(x)
    e = x.numerator.bit_length() - x.denominator.bit_length()
    if Fraction(2) ** e > x:
        e -= 1
    e = max(e, -126)  # subnormal range: fixed scale 2^-149
    m = round(x / Fraction(2) ** (e - 23))  # Fraction.__round__: half to even
    if m == 2 ** 24:
        m, e = 2 ** 23, e + 1
    if e > 127:
        return np.float32(sign * np.inf)
    return np.float32(sign * float(m) * 2.0 ** (e - 23))


def parse_f32(tok: str):
    """Rust's f32 grammar and value; None for a token that is not a float."""
    body = tok[1:] if tok[:1] in "+-" else tok
    if body.lower() in _SPECIAL:
        v = np.float32(np.nan) if body.lower() == "nan" else np.float32(np.inf)
        return -v if tok[:1] == "-" else v
    if not _RUST_FLOAT.match(tok):
        return None
    neg = tok.startswith("-")
    mant, _, exp = body.lower().partition("e")
    ip, _, fp = mant.partition(".")
    digits = (ip + fp) or "0"
    value = Fraction(int(digits)) * Fraction(10) ** (int(exp or "0") - len(fp))
    r = _round_f32(value)
    return -r if neg else r


def tri_tokens(text: str):
    """The reference lexer's tokens, in order."""
    i, n = 0, len(text)
    while True:
        while i < n and text[i] in " \t\\":
            i += 1
        if i < n and text[i] == "#":
            while i < n and text[i] not in "\n\r":
                i += 1
        if i >= n:
            return
        if text[i] in "\n\r":
            yield text[i]
            i += 1
            continue
        j = i
        while j < n and text[j] not in " \t\\\n\r":
            j += 1
        yield text[i:j]
        i = j


def _normalize(v):
    m = np.sqrt(np.float32(np.float32(v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]))
    return np.array([v[0] / m, v[1] / m, v[2] / m], np.float32)


def face_normal(t):
    """normalize(normalize(v2 - v0) x normalize(v1 - v0)) in f32, cglinalg's operation order."""
    v0, v1, v2 = t[0:3], t[3:6], t[6:9]
    a = _normalize(np.array(v2 - v0, np.float32))
    b = _normalize(np.array(v1 - v0, np.float32))
    c = np.array([a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]], np.float32)
    return _normalize(c)


def decode_tri(text: str):
    """TriLoader::load + TriMeshDecoder: (tris [n, 9], normals [n, 9], uvs [n, 6]) float32."""
    toks = list(tri_tokens(text))
    pos, line, tris = 0, 1, []
    while pos < len(toks):
        if toks[pos] == "\n":
            line += 1
            pos += 1
            continue
        tri = []
        for _ in range(9):
            if pos >= len(toks):
                raise DecodeError(line, "EndOfFile")
            tok = toks[pos]
            pos += 1
            if tok == "\n":
                line += 1
            v = parse_f32(tok)
            if v is None:
                raise DecodeError(line, "ExpectedFloat", tok)
            tri.append(v)
        tris.append(tri)
    t = np.array(tris, np.float32).reshape(-1, 9)
    with np.errstate(all="ignore"):
        nrm = np.array([np.tile(face_normal(x), 3) for x in t], np.float32).reshape(-1, 9)
    return t, nrm, np.zeros((len(t), 6), np.float32)


def decode_obj(text: str):
    """First object's faces (fan-split), per-corner normals and texture coordinates, f64 -> f32."""
    v, vt, vn, tris, nrm, uvs = [], [], [], [], [], []
    objects = 0
    for raw in text.split("\n"):
        line = raw.split("#", 1)[0].split()
        if not line:
            continue
        kw = line[0]
        if kw == "o":
            objects += 1
            if objects > 1 or tris:
                break
        elif kw in ("v", "vn"):
            (v if kw == "v" else vn).append([np.float32(float(x)) for x in line[1:4]])
        elif kw == "vt":
            vals = [np.float32(float(x)) for x in line[1:3]]
            vt.append(vals + [np.float32(0.0)] * (2 - len(vals)))
        elif kw == "f":
            corners = []
            for c in line[1:]:
                f = (c.split("/") + ["", ""])[:3]
                idx = []
                for k, (s, pool) in enumerate(zip(f, (v, vt, vn))):
                    if not s:
                        idx.append(None)
                        continue
                    i = int(s)
                    idx.append(i - 1 if i > 0 else len(pool) + i)
                corners.append(idx)
            for k in range(1, len(corners) - 1):
                for vi, ti, ni in (corners[0], corners[k], corners[k + 1]):
                    tris.extend(v[vi])
                    nrm.extend(vn[ni] if ni is not None else [np.float32(0)] * 3)
                    uvs.extend(vt[ti] if ti is not None else [np.float32(0)] * 2)
    return (np.array(tris, np.float32).reshape(-1, 9), np.array(nrm, np.float32).reshape(-1, 9),
            np.array(uvs, np.float32).reshape(-1, 6))
