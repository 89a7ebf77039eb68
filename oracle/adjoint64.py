"""FP64 CPU reference of the differentiable Lambertian render (TEST INFRASTRUCTURE ONLY).

The reference crate has no differentiation and no Lambertian term; what it has is the
barycentric interpolation of per-vertex normals of NormalMappingAccumulator
(bvhtracer/src/renderer.rs:268-272: ``n0 * (1 - u - v) + n1 * u + n2 * v``) and the
Moeller-Trumbore solve of Triangle::intersect (src/geometry/triangle.rs:42-72).  This module
restates the render built on them in float64 -- shading, loss, an analytic adjoint and central
finite differences -- with visibility held fixed (every pixel keeps the triangle it hit in the
forward pass), which is what the CUDA adjoint is checked against.
"""
from __future__ import annotations

import numpy as np


def _solve(o, d, v0, v1, v2):
    """Moeller-Trumbore solve (no inside tests) in float64: t, u, v, determinant a."""
    e1 = v1 - v0
    e2 = v2 - v0
    n = np.cross(d, e2)
    a = np.einsum("ij,ij->i", e1, n)
    f = 1.0 / a
    s = o - v0
    u = f * np.einsum("ij,ij->i", s, n)
    q = np.cross(s, e1)
    v = f * np.einsum("ij,ij->i", d, q)
    t = f * np.einsum("ij,ij->i", e2, q)
    return t, u, v, a, e1, e2


def _shade(o, d, t, u, v, n0, n1, n2, light):
    p = o + d * t[:, None]
    l = light[None, :] - p
    ll = np.linalg.norm(l, axis=1)
    lh = l / ll[:, None]
    w0 = 1.0 - u - v
    n = n0 * w0[:, None] + n1 * u[:, None] + n2 * v[:, None]
    nl = np.linalg.norm(n, axis=1)
    nh = n / nl[:, None]
    c = np.einsum("ij,ij->i", nh, lh)
    return np.maximum(c, 0.0), c, lh, nh, ll, nl


def _pixel_data(rays, prim, verts, faces, vnormals, pix):
    o = rays["origin"][pix].astype(np.float64)
    d = rays["direction"][pix].astype(np.float64)
    f = faces[prim[pix]].astype(np.int64)
    V = verts.astype(np.float64)
    N = vnormals.astype(np.float64)
    return o, d, f, V[f[:, 0]], V[f[:, 1]], V[f[:, 2]], N[f[:, 0]], N[f[:, 1]], N[f[:, 2]]


def render64(rays, prim, verts, faces, vnormals, light):
    """Image in float64 for the hit triangles `prim` (0xFFFFFFFF = miss -> 0)."""
    light = np.asarray(light, np.float64)
    img = np.zeros(len(rays), np.float64)
    pix = np.nonzero(prim != 0xFFFFFFFF)[0]
    o, d, f, v0, v1, v2, n0, n1, n2 = _pixel_data(rays, prim, verts, faces, vnormals, pix)
    t, u, v, _, _, _ = _solve(o, d, v0, v1, v2)
    img[pix] = _shade(o, d, t, u, v, n0, n1, n2, light)[0]
    return img


def loss64(img, target):
    e = img - np.asarray(target, np.float64)
    return float(np.mean(e * e))


def adjoint64(rays, prim, verts, faces, vnormals, light, target, image=None):
    """dLoss/dvertex (float64) for loss = mean((I - target)^2), visibility fixed.  With `image`
    given, the residuals (image - target) use it instead of the float64 intensities (this isolates
    the Jacobian arithmetic of an adjoint from the rounding of its forward pass)."""
    light = np.asarray(light, np.float64)
    target = np.asarray(target, np.float64)
    npix = len(rays)
    grad = np.zeros((len(verts), 3), np.float64)
    pix = np.nonzero(prim != 0xFFFFFFFF)[0]
    o, d, f, v0, v1, v2, n0, n1, n2 = _pixel_data(rays, prim, verts, faces, vnormals, pix)
    t, u, v, a, e1, e2 = _solve(o, d, v0, v1, v2)
    I, c, lh, nh, ll, nl = _shade(o, d, t, u, v, n0, n1, n2, light)
    on = c > 0.0
    Ir = I if image is None else np.asarray(image, np.float64)[pix]
    g = (2.0 / npix) * (Ir - target[pix])
    dn = (lh - c[:, None] * nh) / nl[:, None]
    dl = (nh - c[:, None] * lh) / ll[:, None]
    gt = g * -np.einsum("ij,ij->i", dl, d)
    gu = g * np.einsum("ij,ij->i", dn, n1 - n0)
    gv = g * np.einsum("ij,ij->i", dn, n2 - n0)
    y = (np.cross(e1, e2) * gt[:, None] + np.cross(d, e2) * gu[:, None] + np.cross(e1, d) * gv[:, None]) / a[:, None]
    w = np.stack([1.0 - u - v, u, v], axis=1)
    for k in range(3):
        contrib = -(w[:, k:k + 1] * y)
        contrib[~on] = 0.0
        np.add.at(grad, f[:, k], contrib)
    return grad


def shading_cosine64(rays, prim, verts, faces, vnormals, light):
    """n_hat . l_hat per pixel in float64 (NaN for a miss): the argument of max(0, .)."""
    light = np.asarray(light, np.float64)
    out = np.full(len(rays), np.nan)
    pix = np.nonzero(prim != 0xFFFFFFFF)[0]
    o, d, f, v0, v1, v2, n0, n1, n2 = _pixel_data(rays, prim, verts, faces, vnormals, pix)
    t, u, v, _, _, _ = _solve(o, d, v0, v1, v2)
    out[pix] = _shade(o, d, t, u, v, n0, n1, n2, light)[1]
    return out


def richardson64(rays, prim, verts, faces, vnormals, light, target, coords, eps=1e-3):
    """Central differences with step eps and eps/2 combined as (4 D(eps/2) - D(eps)) / 3, which
    cancels the eps^2 truncation term.  Returns (D(eps), extrapolated)."""
    d1 = finite_differences64(rays, prim, verts, faces, vnormals, light, target, coords, eps)
    d2 = finite_differences64(rays, prim, verts, faces, vnormals, light, target, coords, eps / 2.0)
    return d1, (4.0 * d2 - d1) / 3.0


def finite_differences64(rays, prim, verts, faces, vnormals, light, target, coords, eps=1e-3):
    """Central differences (float64) of the loss for the given (vertex, axis) coordinates, only
    the pixels whose hit triangle uses that vertex change (visibility fixed)."""
    light = np.asarray(light, np.float64)
    target = np.asarray(target, np.float64)
    npix = len(rays)
    V = verts.astype(np.float64)
    hit = np.nonzero(prim != 0xFFFFFFFF)[0]
    fpix = faces[prim[hit]].astype(np.int64)
    out = []
    for vid, axis in coords:
        pix = hit[np.any(fpix == vid, axis=1)]
        vals = []
        for sgn in (+1.0, -1.0):
            Vp = V.copy()
            Vp[vid, axis] += sgn * eps
            o, d, f, v0, v1, v2, n0, n1, n2 = _pixel_data(rays, prim, Vp, faces, vnormals, pix)
            t, u, v, _, _, _ = _solve(o, d, v0, v1, v2)
            I = _shade(o, d, t, u, v, n0, n1, n2, light)[0]
            vals.append(np.sum((I - target[pix]) ** 2))
        out.append((vals[0] - vals[1]) / (2.0 * eps) / npix)
    return np.array(out)
