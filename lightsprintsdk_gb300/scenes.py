"""Seeded synthetic workloads for the collider and the lightmap gather.

Every generator here is bit-reproducible across machines (x86_64 and aarch64):
it uses only integer hashing and IEEE-754 +, -, *, /, sqrt on numpy arrays
(each numpy ufunc rounds once, nothing is fused), in float64, rounded to
float32 at the end.  There is no sin/cos/exp anywhere, because libm results
differ between platforms.  Random directions and shell points are drawn by
rejection from counter-based hashes.

Workloads (the sizes are the ones the collider and gather are measured on):

* ``icosphere_c0``: one displaced geodesic icosphere truncated to 69,451
  triangles; the stand-in for the Stanford-bunny collider benchmark
  (samples/BunnyBenchmark/BunnyBenchmark.cpp:4 quotes 69,451 triangles).
* ``shell_rays``: rays with origins uniform in the volume of the shell
  [1.5 r, 3 r] and directions uniform on the sphere, rayLengthMin=0,
  rayLengthMax=10 r.
* ``interior_c1``: a 20 x 10 x 20 room of tessellated axis-aligned slabs,
  300 seeded boxes and 64 instances of one displaced icosphere
  (12,500 triangles each), about 1.24 M triangles.
* ``camera_rays`` / ``surface_rays`` / ``shadow_rays``: coherent pinhole rays,
  incoherent cosine-hemisphere secondary rays from seeded surface points, and
  any-hit shadow rays from the same points to a point light.

Ray layout (the device input format): float32 array of shape (n, 8) =
(ox, oy, oz, tmin, dx, dy, dz, tmax), i.e. two float4 per ray.
"""
from __future__ import annotations

import numpy as np

M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


# ---------------------------------------------------------------- hashing
def fmix64(k: np.ndarray) -> np.ndarray:
    """MurmurHash3's 64-bit finaliser (public domain), on uint64 arrays."""
    k = np.asarray(k, dtype=np.uint64).copy()
    k ^= k >> np.uint64(33)
    k *= np.uint64(0xFF51AFD7ED558CCD)
    k ^= k >> np.uint64(33)
    k *= np.uint64(0xC4CEB9FE1A85EC53)
    k ^= k >> np.uint64(33)
    return k


def hash_u64(seed: int, stream: int, index) -> np.ndarray:
    """Counter-based 64-bit hash of (seed, stream, index).  The same function
    is restated in C (oracle) and CUDA (gather sampling)."""
    idx = np.asarray(index, dtype=np.uint64)
    key = np.uint64((seed * 0x9E3779B97F4A7C15 + stream * 0xD1B54A32D192ED03) & 0xFFFFFFFFFFFFFFFF)
    return fmix64(fmix64(idx ^ key) + np.uint64(0x632BE59BD9B4E019))


def uniform01(seed: int, stream: int, index) -> np.ndarray:
    """float64 in [0,1) with 53 random bits (exact)."""
    h = hash_u64(seed, stream, index)
    return (h >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def _rejection(n: int, start: int, tries: int, draw, accept, fallback) -> np.ndarray:
    """For rows start..start+n-1, candidate k of row i is draw(i*tries + k)
    (an (m,d) array); the first accepted candidate is kept.  Candidates are
    evaluated in batches (2, then 8 at a time) only for rows still unresolved, so the result
    is that of the full (n, tries) evaluation at a fraction of the cost."""
    fallback = np.asarray(fallback, np.float64)
    out = np.empty((n, fallback.shape[0]), np.float64)
    todo = np.arange(n, dtype=np.int64)
    rows = np.arange(start, start + n, dtype=np.uint64)
    k0 = 0
    while k0 < tries and todo.size:
        step = 2 if k0 == 0 else 8
        kk = np.arange(k0, min(tries, k0 + step), dtype=np.uint64)
        k0 += step
        ids = rows[todo][:, None] * np.uint64(tries) + kk[None, :]
        c = draw(ids)                      # (m, K, d)
        ok = accept(c)                     # (m, K)
        hit = ok.any(axis=1)
        first = ok.argmax(axis=1)
        sel = todo[hit]
        out[sel] = c[np.nonzero(hit)[0], first[hit]]
        todo = todo[~hit]
    out[todo] = fallback
    return out


def unit_vectors(seed: int, stream: int, n: int, start: int = 0, tries: int = 48) -> np.ndarray:
    """n directions uniform on S^2 (float64, unit length), by rejection from
    the cube [-1,1]^3 into the ball 1e-6 < |p|^2 <= 1, then normalisation."""
    def draw(ids):
        return np.stack([uniform01(seed, stream * 3 + a, ids) * 2.0 - 1.0 for a in range(3)], axis=-1)

    def accept(p):
        r2 = (p[..., 0] * p[..., 0] + p[..., 1] * p[..., 1]) + p[..., 2] * p[..., 2]
        return (r2 > 1e-6) & (r2 <= 1.0)

    v = _rejection(n, start, tries, draw, accept, [0.0, 0.0, 1.0])
    l = np.sqrt((v[:, 0] * v[:, 0] + v[:, 1] * v[:, 1]) + v[:, 2] * v[:, 2])
    return v / l[:, None]


def shell_points(seed: int, stream: int, n: int, rmin: float, rmax: float, start: int = 0,
                 tries: int = 48) -> np.ndarray:
    """n points uniform in the volume of the shell rmin <= |p| <= rmax,
    by rejection from the cube [-rmax, rmax]^3."""
    lo2, hi2 = rmin * rmin, rmax * rmax

    def draw(ids):
        return np.stack([(uniform01(seed, stream * 3 + a, ids) * 2.0 - 1.0) * rmax for a in range(3)], axis=-1)

    def accept(p):
        r2 = (p[..., 0] * p[..., 0] + p[..., 1] * p[..., 1]) + p[..., 2] * p[..., 2]
        return (r2 >= lo2) & (r2 <= hi2)

    return _rejection(n, start, tries, draw, accept, [0.0, 0.0, rmax])


# ------------------------------------------------------------ value noise
def value_noise3(p: np.ndarray, seed: int, freq: float) -> np.ndarray:
    """Seeded 3-D value noise in [-1, 1]: lattice values from hash_u64 at
    integer points of p*freq, trilinear interpolation with smoothstep
    weights s(t) = t^2 (3 - 2t)."""
    q = p * freq
    f = np.floor(q)
    t = q - f
    w = t * t * (3.0 - 2.0 * t)
    fi = f.astype(np.int64)

    def lat(ix, iy, iz):
        key = ((ix & 0x1FFFFF).astype(np.uint64) << np.uint64(42)) | \
              ((iy & 0x1FFFFF).astype(np.uint64) << np.uint64(21)) | \
              (iz & 0x1FFFFF).astype(np.uint64)
        return uniform01(seed, 7, key) * 2.0 - 1.0

    x0, y0, z0 = fi[:, 0], fi[:, 1], fi[:, 2]
    res = np.zeros(p.shape[0], np.float64)
    for dx in (0, 1):
        wx = w[:, 0] if dx else 1.0 - w[:, 0]
        for dy in (0, 1):
            wy = w[:, 1] if dy else 1.0 - w[:, 1]
            for dz in (0, 1):
                wz = w[:, 2] if dz else 1.0 - w[:, 2]
                res = res + (wx * wy) * wz * lat(x0 + dx, y0 + dy, z0 + dz)
    return res


# --------------------------------------------------------------- icosphere
def _icosahedron():
    phi = (1.0 + np.sqrt(5.0)) / 2.0
    v = np.array([[-1, phi, 0], [1, phi, 0], [-1, -phi, 0], [1, -phi, 0],
                  [0, -1, phi], [0, 1, phi], [0, -1, -phi], [0, 1, -phi],
                  [phi, 0, -1], [phi, 0, 1], [-phi, 0, -1], [-phi, 0, 1]], np.float64)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
                  [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
                  [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
                  [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], np.int64)
    return v, f


def geodesic_sphere(freq: int):
    """Class-I geodesic subdivision of the icosahedron at frequency `freq`
    (20*freq^2 triangles, 10*freq^2+2 shared vertices, outward CCW winding).
    A point with integer weights (w_a, w_b, w_c) on face (a, b, c) is
    computed from the weights sorted by corner index, so points on shared
    edges are bit-identical from both faces; it is then projected to the
    unit sphere.  Returns float64 vertices (V,3) and int64 triangles (T,3)."""
    iv, faces = _icosahedron()
    key_to_id: dict = {}
    keys = []
    tris = np.empty((20 * freq * freq, 3), np.int64)
    nt = 0
    for a, b, c in faces:
        grid = {}
        for i in range(freq + 1):
            for j in range(freq + 1 - i):
                w = ((int(a), freq - i - j), (int(b), i), (int(c), j))
                key = tuple(sorted(x for x in w if x[1] > 0))
                vid = key_to_id.get(key)
                if vid is None:
                    vid = len(keys)
                    key_to_id[key] = vid
                    keys.append(key)
                grid[(i, j)] = vid
        for i in range(freq):
            for j in range(freq - i):
                tris[nt] = (grid[(i, j)], grid[(i + 1, j)], grid[(i, j + 1)])
                nt += 1
                if i + j < freq - 1:
                    tris[nt] = (grid[(i + 1, j)], grid[(i + 1, j + 1)], grid[(i, j + 1)])
                    nt += 1
    assert nt == tris.shape[0]
    verts = np.zeros((len(keys), 3), np.float64)
    # accumulate in canonical (sorted-corner) order: at most 3 terms
    for slot in range(3):
        idx = np.array([k[slot][0] if len(k) > slot else 0 for k in keys], np.int64)
        wt = np.array([k[slot][1] if len(k) > slot else 0 for k in keys], np.float64)
        verts = verts + wt[:, None] * iv[idx]
    verts = verts / float(freq)
    l = np.sqrt((verts[:, 0] * verts[:, 0] + verts[:, 1] * verts[:, 1]) + verts[:, 2] * verts[:, 2])
    return verts / l[:, None], tris


def displaced_icosphere(freq: int, seed: int, radius: float = 1.0, amp: float = 0.15,
                        noise_freq: float = 2.5):
    """Unit geodesic sphere displaced radially: r * (1 + amp * noise(p))."""
    v, t = geodesic_sphere(freq)
    d = value_noise3(v, seed, noise_freq)
    v = v * (radius * (1.0 + amp * d))[:, None]
    return v, t


def icosphere_c0(seed: int = 0x5EED, ntri: int = 69451):
    """Collider config 0: frequency-59 geodesic sphere (69,620 triangles),
    displaced by 0.15 r value noise, truncated to its first `ntri`
    triangles in generation order (the last face loses 169 triangles, which
    opens a small hole).  Returns float32 vertices (V,3), uint32 indices (T,3)."""
    v, t = displaced_icosphere(59, seed)
    t = t[:ntri]
    return v.astype(np.float32), t.astype(np.uint32)


# ------------------------------------------------------------------- rays
def pack_rays(org: np.ndarray, dirs: np.ndarray, tmin, tmax) -> np.ndarray:
    n = org.shape[0]
    r = np.empty((n, 8), np.float32)
    r[:, 0:3] = org
    r[:, 3] = tmin
    r[:, 4:7] = dirs
    r[:, 7] = tmax
    return r


def shell_rays(n: int, seed: int = 0x5EED, radius: float = 1.0, start: int = 0) -> np.ndarray:
    """Config-0 rays: origins uniform in the shell [1.5r, 3r] (by volume),
    directions uniform on S^2, tmin=0, tmax=10r."""
    o = shell_points(seed, 11, n, 1.5 * radius, 3.0 * radius, start=start)
    d = unit_vectors(seed, 12, n, start=start)
    return pack_rays(o.astype(np.float32), d.astype(np.float32), 0.0, 10.0 * radius)


# -------------------------------------------------------- interior scene
def _box_tris(lo, hi, cell: float):
    """Axis-aligned box [lo, hi] with each of its 6 faces tessellated into a
    grid of about `cell`-sized squares (2 triangles per square), outward
    winding.  Returns float64 vertices and int64 triangles (unshared verts
    per face)."""
    lo = np.asarray(lo, np.float64)
    hi = np.asarray(hi, np.float64)
    vs, ts = [], []
    base = 0
    for axis in range(3):
        u_ax, v_ax = (axis + 1) % 3, (axis + 2) % 3
        nu = max(1, int(np.ceil((hi[u_ax] - lo[u_ax]) / cell - 1e-9)))
        nv = max(1, int(np.ceil((hi[v_ax] - lo[v_ax]) / cell - 1e-9)))
        uu = lo[u_ax] + (hi[u_ax] - lo[u_ax]) * (np.arange(nu + 1) / nu)
        vv = lo[v_ax] + (hi[v_ax] - lo[v_ax]) * (np.arange(nv + 1) / nv)
        gu, gv = np.meshgrid(uu, vv, indexing="ij")
        for side, val in ((0, lo[axis]), (1, hi[axis])):
            p = np.zeros(((nu + 1) * (nv + 1), 3), np.float64)
            p[:, axis] = val
            p[:, u_ax] = gu.ravel()
            p[:, v_ax] = gv.ravel()
            i = np.arange(nu)[:, None] * (nv + 1) + np.arange(nv)[None, :]
            i = i.ravel()
            a, b, c, d = i, i + (nv + 1), i + (nv + 1) + 1, i + 1
            if side == 1:   # normal +axis: (u, v, axis) right-handed -> CCW a,b,c
                t1 = np.stack([a, b, c], 1)
                t2 = np.stack([a, c, d], 1)
            else:
                t1 = np.stack([a, c, b], 1)
                t2 = np.stack([a, d, c], 1)
            vs.append(p)
            ts.append(np.concatenate([t1, t2]) + base)
            base += p.shape[0]
    return np.concatenate(vs), np.concatenate(ts)


def _rand_rotation(seed: int, stream: int, n: int) -> np.ndarray:
    """n rotation matrices from unit quaternions drawn by rejection in the
    4-ball (no trigonometry).  float64 (n,3,3)."""
    def draw(ids):
        return np.stack([uniform01(seed, stream * 4 + a, ids) * 2.0 - 1.0 for a in range(4)], -1)

    def accept(q):
        r2 = ((q[..., 0] * q[..., 0] + q[..., 1] * q[..., 1]) + q[..., 2] * q[..., 2]) + q[..., 3] * q[..., 3]
        return (r2 > 1e-3) & (r2 <= 1.0)

    qq = _rejection(n, 0, 64, draw, accept, [1.0, 0.0, 0.0, 0.0])
    l = np.sqrt(((qq[:, 0] * qq[:, 0] + qq[:, 1] * qq[:, 1]) + qq[:, 2] * qq[:, 2]) + qq[:, 3] * qq[:, 3])
    w, x, y, z = (qq / l[:, None]).T
    m = np.empty((n, 3, 3))
    m[:, 0, 0] = 1 - 2 * (y * y + z * z); m[:, 0, 1] = 2 * (x * y - w * z); m[:, 0, 2] = 2 * (x * z + w * y)
    m[:, 1, 0] = 2 * (x * y + w * z); m[:, 1, 1] = 1 - 2 * (x * x + z * z); m[:, 1, 2] = 2 * (y * z - w * x)
    m[:, 2, 0] = 2 * (x * z - w * y); m[:, 2, 1] = 2 * (y * z + w * x); m[:, 2, 2] = 1 - 2 * (x * x + y * y)
    return m


class Scene:
    """A flattened world-space triangle soup plus its object structure.

    vertices float32 (V,3); indices uint32 (T,3); tri_object int32 (T,)
    (object id of each triangle, objects numbered in generation order);
    object_first_tri int64 (O+1,) prefix offsets; instance_matrices float32
    (I,3,4) for the instanced sphere objects (world = M[:, :3] @ local + M[:, 3])
    and sphere_local (vertices, indices) of the instanced mesh."""

    def __init__(self, vertices, indices, tri_object, object_first_tri, instance_matrices=None,
                 sphere_local=None, instance_object_ids=None):
        self.vertices = vertices
        self.indices = indices
        self.tri_object = tri_object
        self.object_first_tri = object_first_tri
        self.instance_matrices = instance_matrices
        self.sphere_local = sphere_local
        self.instance_object_ids = instance_object_ids

    @property
    def ntri(self) -> int:
        return int(self.indices.shape[0])

    @property
    def nobj(self) -> int:
        return int(self.object_first_tri.shape[0] - 1)


def interior_c1(seed: int = 0xC1, cell: float = 0.125, nboxes: int = 300, ninst: int = 64,
                sphere_freq: int = 25) -> Scene:
    """Collider config 1: room interior x in [-10,10], y in [0,10], z in
    [-10,10] bounded by 0.25-thick axis-aligned slabs tessellated at `cell`
    (floor, four walls, and a ceiling of four slabs around a 6 x 6 skylight); `nboxes` seeded boxes (sides 0.2..1.5) inside; `ninst` instances
    of one displaced icosphere (frequency 25 = 12,500 triangles, radius 1)
    with seeded rotation, scale 0.35..0.8 and position on an 8x8 grid at
    heights 1..8 with jitter.  Objects: 9 slabs, then boxes, then spheres."""
    th = 0.25
    slabs = [
        ((-10 - th, -th, -10 - th), (10 + th, 0.0, 10 + th)),          # floor
        ((-10 - th, 10.0, -10 - th), (10 + th, 10 + th, -3.0)),        # ceiling, around a
        ((-10 - th, 10.0, 3.0), (10 + th, 10 + th, 10 + th)),          #   6 x 6 skylight
        ((-10 - th, 10.0, -3.0), (-3.0, 10 + th, 3.0)),                #   opening over
        ((3.0, 10.0, -3.0), (10 + th, 10 + th, 3.0)),                  #   the centre
        ((-10 - th, 0.0, -10 - th), (-10.0, 10.0, 10 + th)),           # wall -x
        ((10.0, 0.0, -10 - th), (10 + th, 10.0, 10 + th)),             # wall +x
        ((-10.0, 0.0, -10 - th), (10.0, 10.0, -10.0)),                 # wall -z
        ((-10.0, 0.0, 10.0), (10.0, 10.0, 10 + th)),                   # wall +z
    ]
    verts, tris, objs = [], [], []
    base = 0
    oid = 0
    for lo, hi in slabs:
        v, t = _box_tris(lo, hi, cell)
        verts.append(v); tris.append(t + base); objs.append(np.full(t.shape[0], oid, np.int32))
        base += v.shape[0]; oid += 1
    ids = np.arange(nboxes, dtype=np.uint64)
    size = 0.2 + 1.3 * np.stack([uniform01(seed, 20 + a, ids) for a in range(3)], -1)
    cen = np.stack([uniform01(seed, 23, ids) * 18.0 - 9.0,
                    uniform01(seed, 24, ids) * 9.0 + 0.5,
                    uniform01(seed, 25, ids) * 18.0 - 9.0], -1)
    for i in range(nboxes):
        lo = cen[i] - 0.5 * size[i]
        hi = cen[i] + 0.5 * size[i]
        v, t = _box_tris(lo, hi, 1e9)
        verts.append(v); tris.append(t + base); objs.append(np.full(t.shape[0], oid, np.int32))
        base += v.shape[0]; oid += 1
    sv, st = displaced_icosphere(sphere_freq, seed + 1)
    sv32 = sv.astype(np.float32)
    rot = _rand_rotation(seed, 30, ninst)
    iid = np.arange(ninst, dtype=np.uint64)
    scale = 0.35 + 0.45 * uniform01(seed, 31, iid)
    gx = (np.arange(ninst) % 8).astype(np.float64)
    gz = (np.arange(ninst) // 8).astype(np.float64)
    pos = np.stack([gx * 2.4 - 8.4 + (uniform01(seed, 32, iid) - 0.5) * 0.6,
                    1.0 + 7.0 * uniform01(seed, 33, iid),
                    gz * 2.4 - 8.4 + (uniform01(seed, 34, iid) - 0.5) * 0.6], -1)
    mats = np.zeros((ninst, 3, 4), np.float64)
    mats[:, :, :3] = rot * scale[:, None, None]
    mats[:, :, 3] = pos
    mats32 = mats.astype(np.float32)
    inst_obj = []
    svl = sv32.astype(np.float64)
    for i in range(ninst):
        m = mats32[i].astype(np.float64)
        w = ((svl[:, 0:1] * m[None, :, 0] + svl[:, 1:2] * m[None, :, 1]) + svl[:, 2:3] * m[None, :, 2]) + m[None, :, 3]
        verts.append(w); tris.append(st + base); objs.append(np.full(st.shape[0], oid, np.int32))
        inst_obj.append(oid)
        base += w.shape[0]; oid += 1
    V = np.concatenate(verts).astype(np.float32)
    T = np.concatenate(tris).astype(np.uint32)
    O = np.concatenate(objs)
    counts = np.bincount(O, minlength=oid)
    first = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    return Scene(V, T, O, first, mats32, (sv32, st.astype(np.uint32)), np.array(inst_obj, np.int32))


def camera_rays(w: int = 4096, h: int = 4096, eye=(-8.5, 4.0, -8.5), target=(2.0, 3.0, 3.0),
                tan_half_fov: float = 0.7, row_start: int = 0, rows: int | None = None,
                cols=None) -> np.ndarray:
    """Coherent pinhole rays through pixel centres, row-major, tmin=0,
    tmax=1e4.  The camera basis is built without trigonometry.  `cols`
    restricts each row to the given pixel columns (same values as the full
    image's rays at those pixels)."""
    if rows is None:
        rows = h - row_start
    eye = np.array(eye, np.float64)
    fwd = np.array(target, np.float64) - eye
    fwd = fwd / np.sqrt((fwd[0] * fwd[0] + fwd[1] * fwd[1]) + fwd[2] * fwd[2])
    up0 = np.array([0.0, 1.0, 0.0])
    right = np.cross(fwd, up0)
    right = right / np.sqrt((right[0] * right[0] + right[1] * right[1]) + right[2] * right[2])
    up = np.cross(right, fwd)
    ys = (np.arange(row_start, row_start + rows, dtype=np.float64) + 0.5) / h * 2.0 - 1.0
    cx = np.arange(w, dtype=np.float64) if cols is None else np.asarray(cols, np.float64)
    xs = (cx + 0.5) / w * 2.0 - 1.0
    py, px = np.meshgrid(-ys * tan_half_fov, xs * tan_half_fov * (w / h), indexing="ij")
    d = fwd[None, None, :] + px[..., None] * right[None, None, :] + py[..., None] * up[None, None, :]
    d = d.reshape(-1, 3)
    l = np.sqrt((d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2])
    d = d / l[:, None]
    o = np.broadcast_to(eye, d.shape)
    return pack_rays(o.astype(np.float32), d.astype(np.float32), 0.0, 1.0e4)


def _tri_area_cdf(V: np.ndarray, T: np.ndarray):
    a = V[T[:, 0]].astype(np.float64)
    e1 = V[T[:, 1]].astype(np.float64) - a
    e2 = V[T[:, 2]].astype(np.float64) - a
    c = np.cross(e1, e2)
    area = 0.5 * np.sqrt((c[:, 0] * c[:, 0] + c[:, 1] * c[:, 1]) + c[:, 2] * c[:, 2])
    cdf = np.cumsum(area)
    return cdf / cdf[-1], c


def surface_points(scene_v: np.ndarray, scene_t: np.ndarray, n: int, seed: int = 0x5EC, start: int = 0):
    """n seeded surface points, area-weighted over triangles.  Returns
    (points float64 (n,3), unit geometric normals (n,3), triangle ids)."""
    cdf, cr = _tri_area_cdf(scene_v, scene_t)
    ids = np.arange(start, start + n, dtype=np.uint64)
    tri = np.searchsorted(cdf, uniform01(seed, 40, ids), side="right")
    tri = np.minimum(tri, scene_t.shape[0] - 1)
    r1 = uniform01(seed, 41, ids)
    r2 = uniform01(seed, 42, ids)
    s = np.sqrt(r1)
    bu, bv = s * (1.0 - r2), s * r2
    T = scene_t[tri]
    a = scene_v[T[:, 0]].astype(np.float64)
    b = scene_v[T[:, 1]].astype(np.float64)
    c = scene_v[T[:, 2]].astype(np.float64)
    p = a + (b - a) * bu[:, None] + (c - a) * bv[:, None]
    nrm = cr[tri]
    nrm = nrm / np.sqrt((nrm[:, 0] * nrm[:, 0] + nrm[:, 1] * nrm[:, 1]) + nrm[:, 2] * nrm[:, 2])[:, None]
    return p, nrm, tri


def _cosine_dirs(nrm: np.ndarray, seed: int, stream: int, start: int, tries: int = 48) -> np.ndarray:
    """Cosine-weighted directions about unit normals (Malley's method: a
    point uniform in the unit disk lifted to the hemisphere)."""
    n = nrm.shape[0]

    def draw(ids):
        return np.stack([uniform01(seed, stream, ids) * 2.0 - 1.0,
                         uniform01(seed, stream + 1, ids) * 2.0 - 1.0], -1)

    def accept(p):
        return (p[..., 0] * p[..., 0] + p[..., 1] * p[..., 1]) < 0.999999

    xy = _rejection(n, start, tries, draw, accept, [0.0, 0.0])
    z = np.sqrt(1.0 - (xy[:, 0] * xy[:, 0] + xy[:, 1] * xy[:, 1]))
    # tangent frame: t = normalize(orthogonal(n)), b = n x t
    ax = np.abs(nrm[:, 0]) > np.abs(nrm[:, 2])
    t = np.where(ax[:, None], np.stack([-nrm[:, 1], nrm[:, 0], np.zeros(n)], -1),
                 np.stack([np.zeros(n), -nrm[:, 2], nrm[:, 1]], -1))
    t = t / np.sqrt((t[:, 0] * t[:, 0] + t[:, 1] * t[:, 1]) + t[:, 2] * t[:, 2])[:, None]
    b = np.cross(nrm, t)
    d = t * xy[:, 0:1] + b * xy[:, 1:2] + nrm * z[:, None]
    return d / np.sqrt((d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2])[:, None]


def surface_rays(scene_v, scene_t, n: int, seed: int = 0x5EC, start: int = 0, eps: float = 1e-4) -> np.ndarray:
    """Incoherent secondary rays: cosine-hemisphere directions about the
    geometric normal, from seeded surface points; tmin=eps, tmax=1e4."""
    p, nrm, _ = surface_points(scene_v, scene_t, n, seed, start)
    d = _cosine_dirs(nrm, seed, 43, start)
    return pack_rays(p.astype(np.float32), d.astype(np.float32), eps, 1.0e4)


def shadow_rays(scene_v, scene_t, n: int, light=(0.5, 9.0, 0.5), seed: int = 0x5EC, start: int = 0,
                eps: float = 1e-4) -> np.ndarray:
    """Any-hit shadow rays from the same seeded surface points to a point
    light: tmin=eps, tmax = distance to the light minus eps."""
    p, _, _ = surface_points(scene_v, scene_t, n, seed, start)
    d = np.array(light, np.float64)[None, :] - p
    dist = np.sqrt((d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2])
    d = d / dist[:, None]
    r = pack_rays(p.astype(np.float32), d.astype(np.float32), eps, 0.0)
    r[:, 7] = (dist - eps).astype(np.float32)
    return r


# ------------------------------------------------------- lightmap gather
class GatherScene:
    """Inputs of the lightmap final gather on the interior scene.

    albedo float32 (T,3): per-triangle diffuse reflectance, each channel
    uniform in [0.2, 0.8]; tri_atlas int32 (T,): atlas of each triangle;
    uv float32 (T,3,2): lightmap coordinates in [0,1] of the atlas;
    lights: dict with the directional light (direction = where the light
    travels, unit; colour) and the point light (position, colour; irradiance
    colour / (PREVENT_INF + d^2), RRLight.cpp:353-358)."""

    def __init__(self, scene, albedo, tri_atlas, uv, natlas, size, lights):
        self.scene = scene
        self.albedo = albedo
        self.tri_atlas = tri_atlas
        self.uv = uv
        self.natlas = natlas
        self.size = size
        self.lights = lights


def atlas_of_objects(nobj: int, nslab: int, nsphere: int, natlas: int = 256) -> np.ndarray:
    """Object -> atlas: slabs and spheres get an atlas each; the boxes share
    the remaining atlases round robin (box i -> atlas (i mod rest))."""
    a = np.empty(nobj, np.int32)
    nbox = nobj - nslab - nsphere
    a[:nslab] = np.arange(nslab)
    a[nobj - nsphere:] = nslab + np.arange(nsphere)
    rest = natlas - nslab - nsphere
    a[nslab:nslab + nbox] = nslab + nsphere + (np.arange(nbox) % rest)
    return a


def grid_unwrap(tri_atlas: np.ndarray, natlas: int) -> np.ndarray:
    """Per-atlas uniform-grid unwrap: the n triangles of an atlas (in index
    order) fill a g x g grid of square cells, g = ceil(sqrt(ceil(n/2))), two
    triangles per cell: even local index -> lower-left half (corner, +u, +v),
    odd -> upper-right half (opposite corner, -u, -v).  uv in [0,1]."""
    T = tri_atlas.shape[0]
    uv = np.zeros((T, 3, 2), np.float64)
    order = np.argsort(tri_atlas, kind="stable")
    counts = np.bincount(tri_atlas, minlength=natlas)
    starts = np.concatenate([[0], np.cumsum(counts)])
    for a in range(natlas):
        ids = order[starts[a]:starts[a + 1]]
        n = ids.shape[0]
        if n == 0:
            continue
        g = int(np.ceil(np.sqrt(np.ceil(n / 2.0))))
        j = np.arange(n)
        cell = j // 2
        cx = (cell % g).astype(np.float64)
        cy = (cell // g).astype(np.float64)
        lo = np.stack([cx, cy], -1) / g
        c = 1.0 / g
        even = (j % 2) == 0
        p0 = np.where(even[:, None], lo, lo + c)
        p1 = np.where(even[:, None], lo + np.array([c, 0.0]), lo + np.array([0.0, c]))
        p2 = np.where(even[:, None], lo + np.array([0.0, c]), lo + np.array([c, 0.0]))
        uv[ids, 0] = p0
        uv[ids, 1] = p1
        uv[ids, 2] = p2
    return uv.astype(np.float32)


def gather_c2(sc: Scene | None = None, seed: int = 0xC2, natlas: int = 256, size: int = 256) -> GatherScene:
    """Config 2: the interior scene with per-triangle albedo U[0.2,0.8]^3,
    256 atlases of 256 x 256 texels (uniform-grid unwrap), one directional
    light through the skylight and one point light."""
    if sc is None:
        sc = interior_c1()
    T = sc.ntri
    ids = np.arange(T, dtype=np.uint64)
    albedo = np.stack([0.2 + 0.6 * uniform01(seed, 50 + k, ids) for k in range(3)], -1).astype(np.float32)
    nsphere = 0 if sc.instance_object_ids is None else int(sc.instance_object_ids.shape[0])
    atlas_obj = atlas_of_objects(sc.nobj, 9, nsphere, natlas)
    tri_atlas = atlas_obj[sc.tri_object]
    uv = grid_unwrap(tri_atlas, natlas)
    d = np.array([0.25, -1.0, 0.15])
    d = d / np.sqrt((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2])
    lights = {"dir_direction": d.astype(np.float32), "dir_color": np.array([3.0, 2.9, 2.7], np.float32),
              "point_position": np.array([-5.0, 8.0, -5.0], np.float32),
              "point_color": np.array([20.0, 18.0, 15.0], np.float32)}
    return GatherScene(sc, albedo, tri_atlas, uv, natlas, size, lights)


def gather_room(seed: int = 0xC2) -> GatherScene:
    """A small version of the config-2 scene (9,8xx triangles): the same room
    of slabs tessellated at 2.0, 10 boxes, 3 displaced icospheres of
    frequency 4, 16 atlases of 64 x 64 texels, the config-2 lights and
    albedo generator.  Small enough for the reference's own CPU gather to
    cover whole atlases at high quality in seconds."""
    sc = interior_c1(seed=0xC1, cell=2.0, nboxes=10, ninst=3, sphere_freq=4)
    return gather_c2(sc, seed=seed, natlas=16, size=64)


# ------------------------------------------------------- uneven mesh batches
def geodesic_sphere_grid(freq: int):
    """The class-I geodesic sphere of geodesic_sphere(freq) (same vertex
    positions, same 20*freq^2 triangles, outward CCW winding), built with
    array operations: a grid point's identity is the sorted list of its
    (corner, weight) pairs with nonzero weight, encoded as one integer, and
    np.unique merges the copies on shared edges and corners.  Vertex and
    triangle order differ from geodesic_sphere's (vertices in key order,
    triangles face by face, upward ones first)."""
    iv, faces = _icosahedron()
    f = int(freq)
    ii, jj = np.meshgrid(np.arange(f + 1), np.arange(f + 1), indexing="ij")
    inside = ii + jj <= f
    gi, gj = ii[inside], jj[inside]                      # P grid points per face
    P = gi.size
    lut = np.full((f + 1, f + 1), -1, np.int64)
    lut[gi, gj] = np.arange(P)
    w = np.stack([f - gi - gj, gi, gj], -1)              # (P, 3) weights of corners a, b, c
    corners = np.broadcast_to(faces[:, None, :], (20, P, 3))
    weights = np.broadcast_to(w[None], (20, P, 3))
    corners = np.where(weights > 0, corners, 12)         # zero weight -> sentinel, sorts last
    order = np.argsort(corners, axis=-1, kind="stable")
    cs = np.take_along_axis(corners, order, -1)
    ws = np.where(cs == 12, 0, np.take_along_axis(weights, order, -1))
    S = 13 * (f + 1)
    code = cs * (f + 1) + ws
    key = ((code[..., 0] * S + code[..., 1]) * S + code[..., 2]).reshape(-1)
    uniq, first, inv = np.unique(key, return_index=True, return_inverse=True)
    csf = cs.reshape(-1, 3)[first] % 12
    wsf = ws.reshape(-1, 3)[first].astype(np.float64)
    verts = np.zeros((uniq.size, 3), np.float64)
    for slot in range(3):   # canonical (sorted-corner) order: at most 3 terms
        verts = verts + wsf[:, slot:slot + 1] * iv[csf[:, slot]]
    verts = verts / float(f)
    l = np.sqrt((verts[:, 0] * verts[:, 0] + verts[:, 1] * verts[:, 1]) + verts[:, 2] * verts[:, 2])
    verts = verts / l[:, None]
    # triangles of one face in grid-point numbering, then per face
    ui, uj = np.nonzero(np.add.outer(np.arange(f), np.arange(f)) <= f - 1)
    up = np.stack([lut[ui, uj], lut[ui + 1, uj], lut[ui, uj + 1]], -1)
    di, dj = np.nonzero(np.add.outer(np.arange(f), np.arange(f)) <= f - 2)
    down = np.stack([lut[di + 1, dj], lut[di + 1, dj + 1], lut[di, dj + 1]], -1)
    local = np.concatenate([up, down])                   # (f^2, 3)
    tris = (np.arange(20)[:, None, None] * P + local[None]).reshape(-1, 3)
    return verts, inv.reshape(-1)[tris]


def _box_cluster(seed: int, m: int, ntri: int):
    """4..16 seeded boxes in [-1, 1]^3 (sides 0.1..0.8), tessellated so that
    the cluster has about `ntri` triangles (truncated to at most ntri)."""
    nb = 4 + int(hash_u64(seed, 200, m) % np.uint64(13))
    ids = np.arange(nb, dtype=np.uint64) + np.uint64(m) * np.uint64(64)
    size = np.stack([0.1 + 0.7 * uniform01(seed, 201 + a, ids) for a in range(3)], -1)
    ctr = np.stack([-1.0 + (2.0 - size[:, a]) * uniform01(seed, 204 + a, ids) + 0.5 * size[:, a]
                    for a in range(3)], -1)
    area = 2.0 * (size[:, 0] * size[:, 1] + size[:, 1] * size[:, 2] + size[:, 2] * size[:, 0])
    cell = float(np.sqrt(2.0 * area.sum() / max(ntri, 12)))
    vs, ts, base = [], [], 0
    for b in range(nb):
        v, t = _box_tris(ctr[b] - 0.5 * size[b], ctr[b] + 0.5 * size[b], cell)
        vs.append(v)
        ts.append(t + base)
        base += v.shape[0]
    v = np.concatenate(vs)
    t = np.concatenate(ts)[:ntri]
    return v, t


class MeshBatch:
    """Meshes of an uneven batch, concatenated: vertices float32 (V,3),
    indices uint32 (T,3) local to each mesh, vert_off / tri_off uint32
    (M+1,) prefix offsets, kind (M,) 0 = displaced icosphere, 1 = box
    cluster, center float32 (M,3) of each mesh's vertex AABB and radius
    float32 (M,) = half its largest extent (the mesh's size)."""

    def __init__(self, vertices, indices, vert_off, tri_off, kind, center, radius):
        self.vertices = vertices
        self.indices = indices
        self.vert_off = vert_off
        self.tri_off = tri_off
        self.kind = kind
        self.center = center
        self.radius = radius

    @property
    def nmesh(self) -> int:
        return int(self.tri_off.shape[0] - 1)

    def mesh(self, m: int):
        v = self.vertices[self.vert_off[m]:self.vert_off[m + 1]]
        t = self.indices[self.tri_off[m]:self.tri_off[m + 1]]
        return v, t


def log_uniform_counts(seed: int, stream: int, n: int, lo: int, hi: int) -> np.ndarray:
    """n integers log-uniform in [lo, hi]: round(lo * (hi/lo)^u), u from
    uniform01 (the power is taken as exp2 of a float64, the only libm call
    of this module; counts do not need bit reproducibility)."""
    u = uniform01(seed, stream, np.arange(n, dtype=np.uint64))
    return np.clip(np.round(lo * np.exp2(u * np.log2(hi / lo))), lo, hi).astype(np.int64)


def batch_meshes_c3(seed: int = 0xC3, nmesh: int = 512, tri_lo: int = 1000, tri_hi: int = 500_000) -> MeshBatch:
    """Uneven-batching workload: `nmesh` meshes with triangle counts
    log-uniform in [tri_lo, tri_hi]; even-numbered meshes are displaced
    icospheres (frequency ceil(sqrt(n/20)), truncated to n triangles, value
    noise of amplitude 0.15), odd-numbered ones clusters of 4..16 boxes;
    each mesh scaled by 0.5..2 and moved by up to 10 on each axis (its own
    coordinate frame; meshes are independent)."""
    counts = log_uniform_counts(seed, 100, nmesh, tri_lo, tri_hi)
    ids = np.arange(nmesh, dtype=np.uint64)
    scale = 0.5 + 1.5 * uniform01(seed, 101, ids)
    shift = np.stack([-10.0 + 20.0 * uniform01(seed, 102 + a, ids) for a in range(3)], -1)
    vs, ts, kinds = [], [], []
    cache = {}
    for m in range(nmesh):
        n = int(counts[m])
        if m % 2 == 0:
            freq = int(np.ceil(np.sqrt(n / 20.0)))
            if freq not in cache:
                cache[freq] = geodesic_sphere_grid(freq)
            sv, st = cache[freq]
            d = value_noise3(sv, seed + m, 2.5)
            v = sv * (1.0 + 0.15 * d)[:, None]
            t = st[:n]
        else:
            v, t = _box_cluster(seed, m, n)
        vs.append((v * scale[m] + shift[m]).astype(np.float32))
        ts.append(t.astype(np.uint32))
        kinds.append(m % 2)
    vert_off = np.zeros(nmesh + 1, np.int64)
    tri_off = np.zeros(nmesh + 1, np.int64)
    vert_off[1:] = np.cumsum([v.shape[0] for v in vs])
    tri_off[1:] = np.cumsum([t.shape[0] for t in ts])
    lo = np.stack([v.min(0) for v in vs]).astype(np.float64)
    hi = np.stack([v.max(0) for v in vs]).astype(np.float64)
    center = 0.5 * (lo + hi)
    radius = 0.5 * (hi - lo).max(1)
    return MeshBatch(np.concatenate(vs), np.concatenate(ts), vert_off.astype(np.uint32), tri_off.astype(np.uint32),
                     np.array(kinds, np.int32), center.astype(np.float32), radius.astype(np.float32))


def batch_rays(mb: MeshBatch, counts: np.ndarray, seed: int = 0xC3, device: str = "cuda"):
    """Rays of an uneven batch, made with torch on `device` (no host copy of
    the full set): mesh m gets counts[m] rays, the first half coherent
    (a pinhole camera 3 r from its centre, looking at it through a
    ceil(sqrt(k)) x ceil(sqrt(k)) image, half-angle tangent 0.4), the rest
    incoherent (origins uniform in the shell [1.5 r, 3 r] around the centre,
    directions uniform on the sphere); tmin 0, tmax 10 r.  Seeded with a
    torch.Generator; reproducible for one torch build and device type.
    Returns (rays float32 (n, 8), ray_off int64 (M+1,) host array)."""
    import torch
    counts = np.asarray(counts, np.int64)
    M = mb.nmesh
    off = np.zeros(M + 1, np.int64)
    off[1:] = np.cumsum(counts)
    n = int(off[-1])
    dev = torch.device(device)
    g = torch.Generator(device=dev)
    g.manual_seed(seed)
    cnt = torch.from_numpy(counts).to(dev)
    mesh = torch.repeat_interleave(torch.arange(M, device=dev), cnt)
    j = torch.arange(n, device=dev) - torch.from_numpy(off[:-1]).to(dev)[mesh]
    half = (cnt // 2)[mesh]
    coherent = j < half
    ctr = torch.from_numpy(mb.center).to(dev)[mesh]
    rad = torch.from_numpy(mb.radius).to(dev)[mesh]
    # per-mesh camera
    fwd = torch.randn((M, 3), generator=g, device=dev)
    fwd = fwd / fwd.norm(dim=1, keepdim=True)
    up0 = torch.where(fwd[:, 1:2].abs() < 0.9, torch.tensor([0.0, 1.0, 0.0], device=dev),
                      torch.tensor([1.0, 0.0, 0.0], device=dev))
    right = torch.linalg.cross(fwd, up0)
    right = right / right.norm(dim=1, keepdim=True)
    up = torch.linalg.cross(right, fwd)
    w = torch.ceil(torch.sqrt(torch.clamp(cnt // 2, min=1).double())).long()[mesh]
    px = (j % w).float()
    py = (j // w).float()
    sx = (2.0 * (px + 0.5) / w.float() - 1.0) * 0.4
    sy = (2.0 * (py + 0.5) / w.float() - 1.0) * 0.4
    dc = fwd[mesh] + sx[:, None] * right[mesh] + sy[:, None] * up[mesh]
    dc = dc / dc.norm(dim=1, keepdim=True)
    oc = ctr - 3.0 * rad[:, None] * fwd[mesh]
    # incoherent: shell origins, uniform directions
    di = torch.randn((n, 3), generator=g, device=dev)
    di = di / di.norm(dim=1, keepdim=True).clamp_min(1e-12)
    u = torch.rand((n,), generator=g, device=dev)
    rr = torch.pow(1.5 ** 3 + u * (3.0 ** 3 - 1.5 ** 3), 1.0 / 3.0)
    pdir = torch.randn((n, 3), generator=g, device=dev)
    pdir = pdir / pdir.norm(dim=1, keepdim=True).clamp_min(1e-12)
    oi = ctr + (rr * rad)[:, None] * pdir
    rays = torch.empty((n, 8), dtype=torch.float32, device=dev)
    c = coherent[:, None]
    rays[:, 0:3] = torch.where(c, oc, oi)
    rays[:, 3] = 0.0
    rays[:, 4:7] = torch.where(c, dc, di)
    rays[:, 7] = 10.0 * rad
    return rays, off
