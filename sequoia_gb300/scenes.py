"""Seeded synthetic scenes and ray sets for the benchmark configurations.

No dataset is shipped with Sequoia (its published run used a bunny OBJ that
is not in the repository), so every input here is generated from a seed.
Triangles are float32 arrays of shape (n, 9): v0, v1, v2.

  displaced_icosphere(level=6, seed=1)   81,920 tris   (config "small")
  gaussian_soup(2_000_000, 64, seed=2)   2M tris       (config "large")
  heightfield(2048, 1024, seed=3)        4,194,304 tris (precision config)
  mesh_batch(256, seed=4000)             ~12M tris over 256 meshes
  gaussian_soup(8_000_000, 256, seed=5)  8M tris       (incoherent stress)
"""
from __future__ import annotations

import functools
import math

import numpy as np

__all__ = [
    "icosphere", "displaced_icosphere", "gaussian_soup", "heightfield",
    "scene_box", "write_obj", "read_obj", "random_rays", "bounce_rays",
    "batch_sizes", "mesh_batch", "CONFIGS",
]


@functools.lru_cache(maxsize=8)
def _icosphere_cached(level: int):
    v, f = _icosphere(level)
    v.setflags(write=False)
    f.setflags(write=False)
    return v, f


def icosphere(level: int):
    """Unit icosphere: returns (vertices float64 (v,3), faces int64 (f,3))."""
    v, f = _icosphere_cached(level)
    return v.copy(), f.copy()


def _icosphere(level: int):
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = np.array([(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0),
                  (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
                  (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)], dtype=np.float64)
    f = np.array([(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11),
                  (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6), (7, 1, 8),
                  (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9),
                  (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)], dtype=np.int64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    for _ in range(level):
        a, b, c = f[:, 0], f[:, 1], f[:, 2]
        e = np.stack([np.stack([a, b], 1), np.stack([b, c], 1), np.stack([c, a], 1)], 1)
        es = np.sort(e.reshape(-1, 2), axis=1)
        uniq, inv = np.unique(es, axis=0, return_inverse=True)
        mid = v[uniq[:, 0]] + v[uniq[:, 1]]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        m = inv.reshape(-1, 3) + len(v)
        ab, bc, ca = m[:, 0], m[:, 1], m[:, 2]
        v = np.concatenate([v, mid])
        f = np.concatenate([np.stack([a, ab, ca], 1), np.stack([b, bc, ab], 1),
                            np.stack([c, ca, bc], 1), np.stack([ab, bc, ca], 1)])
    return v, f


def displaced_icosphere(level: int = 6, seed: int = 1, amplitude: float = 0.05,
                        return_mesh: bool = False):
    """Icosphere with radius 1 + amplitude * sum_k sin(a_k x + b_k y + c_k z + phi_k),
    k = 1..4, a, b, c ~ U[1, 4], phi ~ U[0, 2 pi)."""
    rng = np.random.default_rng(seed)
    a = rng.uniform(1.0, 4.0, 4)
    b = rng.uniform(1.0, 4.0, 4)
    c = rng.uniform(1.0, 4.0, 4)
    phi = rng.uniform(0.0, 2.0 * math.pi, 4)
    v, f = icosphere(level)
    s = np.zeros(len(v))
    for k in range(4):
        s += np.sin(a[k] * v[:, 0] + b[k] * v[:, 1] + c[k] * v[:, 2] + phi[k])
    v = (v * (1.0 + amplitude * s)[:, None]).astype(np.float32)
    tris = v[f].reshape(-1, 9)
    if return_mesh:
        return np.ascontiguousarray(tris), v, f
    return np.ascontiguousarray(tris)


def _random_rotations(rng, n):
    q = rng.standard_normal((n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    r = np.empty((n, 3, 3))
    r[:, 0, 0] = 1 - 2 * (y * y + z * z); r[:, 0, 1] = 2 * (x * y - z * w); r[:, 0, 2] = 2 * (x * z + y * w)
    r[:, 1, 0] = 2 * (x * y + z * w); r[:, 1, 1] = 1 - 2 * (x * x + z * z); r[:, 1, 2] = 2 * (y * z - x * w)
    r[:, 2, 0] = 2 * (x * z - y * w); r[:, 2, 1] = 2 * (y * z + x * w); r[:, 2, 2] = 1 - 2 * (x * x + y * y)
    return r


def gaussian_soup(n: int = 2_000_000, clusters: int = 64, seed: int = 2,
                  edge_mu: float = math.log(0.02), edge_sigma: float = 0.5,
                  chunk: int = 1 << 21):
    """Triangle soup: centroids from a mixture of `clusters` isotropic Gaussians
    (centres U[-10, 10]^3, sigma U[0.2, 2], component uniform); equilateral
    triangles with lognormal edge length and a uniformly random orientation."""
    rng = np.random.default_rng(seed)
    centres = rng.uniform(-10.0, 10.0, (clusters, 3))
    sigma = rng.uniform(0.2, 2.0, clusters)
    out = np.empty((n, 9), dtype=np.float32)
    ang = np.array([0.0, 2.0 * math.pi / 3.0, 4.0 * math.pi / 3.0])
    local = np.stack([np.cos(ang), np.sin(ang), np.zeros(3)], 1)  # (3 verts, xyz)
    for s in range(0, n, chunk):
        m = min(chunk, n - s)
        comp = rng.integers(0, clusters, m)
        cen = centres[comp] + sigma[comp, None] * rng.standard_normal((m, 3))
        edge = rng.lognormal(edge_mu, edge_sigma, m)
        rot = _random_rotations(rng, m)
        circ = edge / math.sqrt(3.0)
        verts = np.einsum("nij,kj->nki", rot, local) * circ[:, None, None] + cen[:, None, :]
        out[s:s + m] = verts.reshape(m, 9).astype(np.float32)
    return out


def _value_noise(rng, x, z, octaves=8, base_freq=4):
    total = np.zeros_like(x)
    amp, norm = 1.0, 0.0
    for o in range(octaves):
        freq = base_freq * (2 ** o)
        lat = rng.uniform(-1.0, 1.0, (freq + 2, 2 * freq + 2))
        gx = (x + 1.0) * 0.5 * (2 * freq)   # x in [-1, 1] -> [0, 2 freq]
        gz = (z + 0.5) * freq               # z in [-0.5, 0.5] -> [0, freq]
        ix = np.clip(np.floor(gx).astype(np.int64), 0, 2 * freq)
        iz = np.clip(np.floor(gz).astype(np.int64), 0, freq)
        fx = gx - ix
        fz = gz - iz
        sx = fx * fx * (3 - 2 * fx)
        sz = fz * fz * (3 - 2 * fz)
        v00 = lat[iz, ix]; v01 = lat[iz, ix + 1]
        v10 = lat[iz + 1, ix]; v11 = lat[iz + 1, ix + 1]
        v0 = v00 + (v01 - v00) * sx
        v1 = v10 + (v11 - v10) * sx
        total += amp * (v0 + (v1 - v0) * sz)
        norm += amp
        amp *= 0.5
    return total / norm


def heightfield(nx: int = 2048, nz: int = 1024, seed: int = 3, amplitude: float = 0.1):
    """Height-field terrain over x in [-1, 1], z in [-0.5, 0.5]: nx * nz quads,
    two triangles each; height = amplitude * extent * 8-octave value noise."""
    rng = np.random.default_rng(seed)
    xs = np.linspace(-1.0, 1.0, nx + 1)
    zs = np.linspace(-0.5, 0.5, nz + 1)
    x, z = np.meshgrid(xs, zs)               # (nz+1, nx+1)
    y = amplitude * 2.0 * _value_noise(rng, x, z)
    v = np.stack([x, y, z], -1).astype(np.float32)
    v00 = v[:-1, :-1].reshape(-1, 3); v10 = v[:-1, 1:].reshape(-1, 3)
    v01 = v[1:, :-1].reshape(-1, 3); v11 = v[1:, 1:].reshape(-1, 3)
    t1 = np.concatenate([v00, v10, v11], 1)
    t2 = np.concatenate([v00, v11, v01], 1)
    tris = np.empty((2 * len(t1), 9), dtype=np.float32)
    tris[0::2] = t1
    tris[1::2] = t2
    return tris


def scene_box(tris):
    v = tris.reshape(-1, 3)
    return v.min(0), v.max(0)


def write_obj(path, vertices, faces):
    """OBJ with %.9g coordinates, which round-trip float32 exactly through
    the reference loader's atof -> float (src/main.cpp:137-139)."""
    with open(path, "w") as fh:
        for p in np.asarray(vertices, dtype=np.float32):
            fh.write("v %.9g %.9g %.9g\n" % (p[0], p[1], p[2]))
        for t in np.asarray(faces):
            fh.write("f %d %d %d\n" % (t[0] + 1, t[1] + 1, t[2] + 1))


def read_obj(path):
    """Minimal OBJ reader (v / f, quads split, negative indices)."""
    vs, fs = [], []
    with open(path) as fh:
        for line in fh:
            tok = line.split()
            if not tok:
                continue
            if tok[0] == "v":
                vs.append([float(t) for t in tok[1:4]])
            elif tok[0] == "f":
                idx = [int(t.split("/")[0]) for t in tok[1:]]
                idx = [i - 1 if i > 0 else len(vs) + i for i in idx]
                fs.append(idx[:3])
                if len(idx) > 3:
                    fs.append([idx[0], idx[2], idx[3]])
    v = np.array(vs, dtype=np.float32)
    return np.ascontiguousarray(v[np.array(fs)].reshape(-1, 9))


def random_rays(n: int, lo, hi, seed: int = 5, tmax: float = 3.4e38):
    """Origins uniform in the box [lo, hi], directions uniform on the unit
    sphere; returns float32 (n, 8) {o, tmin, d, tmax}."""
    rng = np.random.default_rng(seed)
    r = np.empty((n, 8), dtype=np.float32)
    lo = np.asarray(lo, np.float64); hi = np.asarray(hi, np.float64)
    r[:, 0:3] = rng.uniform(lo, hi, (n, 3))
    d = rng.standard_normal((n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r[:, 3] = 0.0
    r[:, 4:7] = d
    r[:, 7] = tmax
    return r


def pinhole_rays(w: int, h: int, eye, target, up, vfov: float):
    """Pinhole camera rays, one per pixel centre, row after row, as float32
    (n, 8) records {origin, tmin = 0, direction, tmax = FLT_MAX}: the
    library's pinhole (basis in double, rounded to float; each float32
    operation rounded once, in the kernels' order)."""
    f = np.asarray(target, np.float64) - np.asarray(eye, np.float64)
    f /= np.sqrt((f * f).sum())
    upv = np.asarray(up, np.float64)
    r = np.array([f[1] * upv[2] - f[2] * upv[1], f[2] * upv[0] - f[0] * upv[2], f[0] * upv[1] - f[1] * upv[0]])
    r /= np.sqrt((r * r).sum())
    u = np.array([r[1] * f[2] - r[2] * f[1], r[2] * f[0] - r[0] * f[2], r[0] * f[1] - r[1] * f[0]])
    th = math.tan(vfov * math.pi / 360.0)
    f32 = np.float32
    fb, rb, ub = f.astype(f32), r.astype(f32), u.astype(f32)
    sx, sy = f32(th * w / h), f32(th)
    px = ((np.arange(w, dtype=f32) + f32(0.5)) / f32(w)) * f32(2) - f32(1)
    py = ((np.arange(h, dtype=f32) + f32(0.5)) / f32(h)) * f32(2) - f32(1)
    px, py = np.meshgrid(px * sx, py * sy)
    px, py = px.ravel(), py.ravel()
    d = np.stack([(fb[k] + px * rb[k]) + py * ub[k] for k in range(3)], 1)
    l2 = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]
    d = d / np.sqrt(l2)[:, None]
    out = np.empty((w * h, 8), np.float32)
    out[:, 0:3] = np.asarray(eye, np.float32)
    out[:, 3] = 0.0
    out[:, 4:7] = d
    out[:, 7] = np.finfo(np.float32).max
    return out


def _hash_u32(x):
    x = x.astype(np.uint64)
    x = (x ^ (x >> np.uint64(16))) * np.uint64(0x7FEB352D) & np.uint64(0xFFFFFFFF)
    x = (x ^ (x >> np.uint64(15))) * np.uint64(0x846CA68B) & np.uint64(0xFFFFFFFF)
    x = x ^ (x >> np.uint64(16))
    return x & np.uint64(0xFFFFFFFF)


def bounce_rays(tris, rays, ids, ts, seed: int = 3, eps: float = 1e-4):
    """One cosine-weighted diffuse bounce per hit: origin at the hit point
    pushed eps along the facing normal; two uniforms per pixel from a hash of
    (seed xor pixel index).  Returns (bounce rays float32 (m, 8), pixel index)."""
    hit = np.nonzero(ids != 0xFFFFFFFF)[0]
    r = rays[hit].astype(np.float64)
    t = ts[hit].astype(np.float64)
    tv = tris[ids[hit]].astype(np.float64).reshape(-1, 3, 3)
    nrm = np.cross(tv[:, 1] - tv[:, 0], tv[:, 2] - tv[:, 0])
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    flip = np.sum(nrm * r[:, 4:7], 1) > 0
    nrm[flip] *= -1
    p = r[:, 0:3] + t[:, None] * r[:, 4:7] + eps * nrm
    h1 = _hash_u32(np.uint64(seed) ^ hit.astype(np.uint64))
    h2 = _hash_u32(h1 ^ np.uint64(0x9E3779B9))
    u1 = (h1.astype(np.float64) + 0.5) / 4294967296.0
    u2 = (h2.astype(np.float64) + 0.5) / 4294967296.0
    rad = np.sqrt(u1)
    phi = 2 * math.pi * u2
    lx, ly, lz = rad * np.cos(phi), rad * np.sin(phi), np.sqrt(1 - u1)
    a = np.where(np.abs(nrm[:, 0:1]) > 0.9, np.array([[0.0, 1.0, 0.0]]), np.array([[1.0, 0.0, 0.0]]))
    tx = np.cross(a, nrm)
    tx /= np.linalg.norm(tx, axis=1, keepdims=True)
    ty = np.cross(nrm, tx)
    d = lx[:, None] * tx + ly[:, None] * ty + lz[:, None] * nrm
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    out = np.empty((len(hit), 8), dtype=np.float32)
    out[:, 0:3] = p
    out[:, 3] = 0.0
    out[:, 4:7] = d
    out[:, 7] = 3.4e38
    return out, hit


def batch_sizes(total: int = 1 << 24, count: int = 64, lo: int = 16 << 10,
                hi: int = 1 << 20, seed: int = 5):
    """`count` batch sizes log-uniform in [lo, hi], scaled to sum to `total`;
    the last batch absorbs the rounding."""
    rng = np.random.default_rng(seed + 1)
    s = np.exp(rng.uniform(math.log(lo), math.log(hi), count))
    s = np.floor(s / s.sum() * total).astype(np.int64)
    s[-1] += total - s.sum()
    return s


def mesh_batch(count: int = 256, seed: int = 4000, lo: int = 1000, hi: int = 200_000):
    """`count` independent meshes (displaced icosphere or Gaussian soup, chosen
    by the per-mesh seed) with triangle counts log-uniform in [lo, hi], and a
    square primary-ray tile side log-uniform in [64, 512] per mesh.  An
    icosphere mesh is the first n triangles of the smallest subdivision level
    that has at least n."""
    meshes, tiles = [], []
    for i in range(count):
        rng = np.random.default_rng(seed + i)
        n = int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))
        side = int(round(math.exp(rng.uniform(math.log(64), math.log(512)))))
        if rng.uniform() < 0.5:
            # the first n triangles of the smallest icosphere level with at least n
            level = 0
            while 20 * 4 ** level < n:
                level += 1
            tris = np.ascontiguousarray(displaced_icosphere(level, seed=seed + i)[:n])
        else:
            tris = gaussian_soup(n, clusters=8, seed=seed + i)
        meshes.append(tris)
        tiles.append(side)
    return meshes, tiles


# Camera and size presets of the five benchmark configurations.
CONFIGS = {
    "icosphere_l6": dict(eye=(0.0, 0.0, 3.0), target=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0),
                         vfov=60.0, width=1920, height=1080),
    "soup_2m": dict(eye=(0.0, 0.0, -40.0), target=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0),
                    vfov=60.0, width=3840, height=2160),
    "terrain_4m": dict(eye=(0.0, 0.6, -1.2), target=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0),
                       vfov=60.0, width=1920, height=1080),
}
