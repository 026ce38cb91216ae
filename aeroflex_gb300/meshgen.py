"""Synthetic mesh generators for the rans residual workloads, plus a gmsh 4.1
ASCII writer whose output the library's loader (and AeroFLEX's own reader,
src/rans/include/rans/mesh.h:457-738) parse back into the same cells.

A mesh is a dict of numpy arrays:
  x, y     node coordinates (float64)
  cells    (N, 4) int32 node indices, -1 in slot 3 for a triangle
  bedges   (B, 2) int32 node indices of boundary edges
  bpatch   (B,)   int32 index into ``names``
  names    list of boundary patch names
"""
import math

import numpy as np



def _libm(fn, x):
    """fn (a function of Python's math module, i.e. the C library) applied
    element by element.  NumPy's own vectorised transcendental functions
    differ between CPU architectures in the last bit; the C library's agree,
    so meshes generated on different hosts are bit-identical."""
    x = np.asarray(x, np.float64)
    return np.fromiter((fn(v) for v in x.ravel().tolist()), np.float64, count=x.size).reshape(x.shape)


def _cos(x):
    return _libm(math.cos, x)


def _sin(x):
    return _libm(math.sin, x)


def _pow(base, k):
    """base ** k for each (integer) exponent k, by the C library's pow."""
    return _libm(lambda e: math.pow(base, e), np.asarray(k, np.float64))


def naca4_thickness(x, t):
    """NACA 4-digit half thickness with the closed trailing edge (-0.1036)."""
    x = np.asarray(x, np.float64)
    return 5.0 * t * (0.2969 * np.sqrt(x) - 0.1260 * x - 0.3516 * x * x + 0.2843 * _libm(lambda v: math.pow(v, 3), x)
                      - 0.1036 * _libm(lambda v: math.pow(v, 4), x))


def naca4_surface(n_surf, m=0.0, p=0.4, t=0.12):
    """``n_surf`` distinct surface points, counter-clockwise from the trailing
    edge over the upper surface, cosine-clustered at both edges."""
    j = np.arange(n_surf)
    beta = 2.0 * np.pi * j / n_surf
    xc = 0.5 * (1.0 + _cos(beta))
    yt = naca4_thickness(xc, t)
    if m > 0.0:
        yc = np.where(xc < p, m / p ** 2 * (2 * p * xc - xc ** 2),
                      m / (1 - p) ** 2 * ((1 - 2 * p) + 2 * p * xc - xc ** 2))
        dyc = np.where(xc < p, 2 * m / p ** 2 * (p - xc), 2 * m / (1 - p) ** 2 * (p - xc))
    else:
        yc = np.zeros_like(xc)
        dyc = np.zeros_like(xc)
    th = _libm(math.atan, dyc)
    sgn = np.where(j <= n_surf // 2, 1.0, -1.0)
    x = xc - sgn * yt * _sin(th)
    y = yc + sgn * yt * _cos(th)
    # exact closure at the trailing edge and leading edge
    x[0], y[0] = 1.0, 0.0
    return x, y


def airfoil_omesh(n_surf=128, n_rad=64, r_far=20.0, growth=None, first=2e-3, m=0.0, p=0.4, t=0.12, split=True,
                  fade=1):
    """O-mesh around a NACA 4-digit airfoil of chord 1.

    ``n_surf`` distinct surface nodes, ``n_rad + 1`` node layers whose
    spacing grows geometrically out to a circle of radius ``r_far`` chords
    centred at mid-chord; the ratio is ``growth`` if given, else the one that
    makes the first layer ``first`` chords thick.  Grid lines leave the
    surface along its normal and blend linearly (in the layer coordinate)
    into uniformly spaced points on the far-field circle; the normal offset
    fades as (1 - s)^fade in the layer coordinate s (fade = 2 keeps the
    outer layers of fine meshes from folding).  Each quad is split into two
    triangles along a fixed diagonal when ``split``.  Patches: "wall"
    (airfoil) and "farfield" (outer circle).
    """
    sx, sy = naca4_surface(n_surf, m, p, t)
    ang = 2.0 * np.pi * np.arange(n_surf) / n_surf
    fx = 0.5 + r_far * _cos(ang)
    fy = r_far * _sin(ang)
    # outward normals: rotate the central-difference tangent (CCW surface -> outward = (ty, -tx))
    tx = np.roll(sx, -1) - np.roll(sx, 1)
    ty = np.roll(sy, -1) - np.roll(sy, 1)
    tn = np.sqrt(tx * tx + ty * ty)
    nx_, ny_ = ty / tn, -tx / tn
    if growth is None:
        # geometric ratio r with r_far*(r - 1)/(r^n - 1) = first (bisection)
        lo, hi = 1.0 + 1e-9, 2.0
        for _ in range(200):
            mid = 0.5 * (lo + hi)
            h1 = r_far * (mid - 1.0) / (mid ** n_rad - 1.0)
            lo, hi = (lo, mid) if h1 < first else (mid, hi)
        growth = 0.5 * (lo + hi)
    k = np.arange(n_rad + 1)
    s = (_pow(growth, k) - 1.0) / (math.pow(growth, n_rad) - 1.0)
    S = s[:, None]
    if fade == 1:
        X = (1.0 - S) * (sx[None, :] + r_far * S * nx_[None, :]) + S * fx[None, :]
        Y = (1.0 - S) * (sy[None, :] + r_far * S * ny_[None, :]) + S * fy[None, :]
    else:
        F = (1.0 - S) ** fade * r_far * S
        X = (1.0 - S) * sx[None, :] + F * nx_[None, :] + S * fx[None, :]
        Y = (1.0 - S) * sy[None, :] + F * ny_[None, :] + S * fy[None, :]
    x = X.reshape(-1)
    y = Y.reshape(-1)

    def nid(kk, jj):
        return kk * n_surf + (jj % n_surf)

    kk, jj = np.meshgrid(np.arange(n_rad), np.arange(n_surf), indexing="ij")
    a = nid(kk, jj)
    b = nid(kk, jj + 1)
    c = nid(kk + 1, jj + 1)
    d = nid(kk + 1, jj)
    if split:
        # diagonals alternate in a checkerboard: a one-way split biases the
        # Green-Gauss reconstruction and stalls the explicit scheme
        neg = np.full_like(a, -1)
        alt = ((kk + jj) % 2 == 1)[..., None]
        t1 = np.where(alt, np.stack([a, b, d, neg], -1), np.stack([a, b, c, neg], -1)).reshape(-1, 4)
        t2 = np.where(alt, np.stack([b, c, d, neg], -1), np.stack([a, c, d, neg], -1)).reshape(-1, 4)
        cells = np.stack([t1, t2], 1).reshape(-1, 4)
    else:
        cells = np.stack([a, b, c, d], -1).reshape(-1, 4)
    js = np.arange(n_surf)
    wall = np.stack([nid(0, js), nid(0, js + 1)], -1)
    far = np.stack([nid(n_rad, js), nid(n_rad, js + 1)], -1)
    bedges = np.concatenate([wall, far]).astype(np.int32)
    bpatch = np.concatenate([np.zeros(n_surf), np.ones(n_surf)]).astype(np.int32)
    return dict(x=x, y=y, cells=cells.astype(np.int32), bedges=bedges, bpatch=bpatch, names=["wall", "farfield"])


def channel(nx=2048, ny=1024, jitter=0.2, seed=1, shuffle_seed=2):
    """Unit-square channel triangulated from ``nx`` x ``ny`` quads (2 triangles
    each).  Interior nodes are jittered by uniform +-``jitter``*h (seed
    ``seed``) and the cells shuffled (seed ``shuffle_seed``; None keeps the
    generator order).  Patches: "farfield" (left and right) and "wall"
    (bottom and top)."""
    xs = np.linspace(0.0, 1.0, nx + 1)
    ys = np.linspace(0.0, 1.0, ny + 1)
    X, Y = np.meshgrid(xs, ys, indexing="ij")  # node (i, j) -> i*(ny+1) + j
    if jitter:
        rng = np.random.default_rng(seed)
        jx = rng.uniform(-jitter, jitter, X.shape) / nx
        jy = rng.uniform(-jitter, jitter, Y.shape) / ny
        inner = np.zeros(X.shape, bool)
        inner[1:-1, 1:-1] = True
        X = np.where(inner, X + jx, X)
        Y = np.where(inner, Y + jy, Y)
    x = X.reshape(-1)
    y = Y.reshape(-1)
    ii, jj = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    a = ii * (ny + 1) + jj
    b = (ii + 1) * (ny + 1) + jj
    c = (ii + 1) * (ny + 1) + jj + 1
    d = ii * (ny + 1) + jj + 1
    neg = np.full(a.shape, -1)
    t1 = np.stack([a, b, c, neg], -1).reshape(-1, 4)
    t2 = np.stack([a, c, d, neg], -1).reshape(-1, 4)
    cells = np.stack([t1, t2], 1).reshape(-1, 4).astype(np.int32)
    if shuffle_seed is not None:
        perm = np.random.default_rng(shuffle_seed).permutation(len(cells))
        cells = cells[perm]
    i = np.arange(nx)
    j = np.arange(ny)
    left = np.stack([j, j + 1], -1)
    right = np.stack([nx * (ny + 1) + j, nx * (ny + 1) + j + 1], -1)
    bottom = np.stack([i * (ny + 1), (i + 1) * (ny + 1)], -1)
    top = np.stack([i * (ny + 1) + ny, (i + 1) * (ny + 1) + ny], -1)
    bedges = np.concatenate([left, right, bottom, top]).astype(np.int32)
    bpatch = np.concatenate([np.zeros(2 * ny), np.ones(2 * nx)]).astype(np.int32)
    return dict(x=x, y=y, cells=cells, bedges=bedges, bpatch=bpatch, names=["farfield", "wall"])


def cell_centroids(m):
    """Vertex-mean centroids in the order mesh.h:384-396 forms them."""
    cells = m["cells"]
    tri = cells[:, 3] < 0
    n = np.where(tri, 3.0, 4.0)
    cx = np.zeros(len(cells))
    cy = np.zeros(len(cells))
    for j in range(4):
        idx = np.where(cells[:, j] >= 0, cells[:, j], 0)
        use = (j < 3) | ~tri
        cx = np.where(use, cx + m["x"][idx] / n, cx)
        cy = np.where(use, cy + m["y"][idx] / n, cy)
    return cx, cy


def density_bump_state(m, mach=0.3, amp=0.05, width=0.1, center=(0.5, 0.5), gamma=1.4, R=0.71428571428):
    """Uniform freestream at ``mach`` (p = 1, T = 1, angle 0) with the density
    multiplied by 1 + amp*exp(-|x - center|^2 / width^2) at uniform p and u.
    Returns the AoS state [rho, rhou, rhov, rhoE] per real cell (N*4)."""
    cx, cy = cell_centroids(m)
    c = math.sqrt(gamma * R * 1.0)
    u = mach * c
    rho_inf = 1.0 / (R * 1.0)
    r2 = (cx - center[0]) ** 2 + (cy - center[1]) ** 2
    rho = rho_inf * (1.0 + amp * _libm(math.exp, -r2 / width ** 2))
    q = np.empty((len(cx), 4))
    q[:, 0] = rho
    q[:, 1] = rho * u
    q[:, 2] = 0.0
    q[:, 3] = 1.0 / (gamma - 1.0) + 0.5 * rho * u * u
    return q.reshape(-1)


def write_gmsh(path, m):
    """Write ``m`` as gmsh 4.1 ASCII: one curve entity per boundary patch and
    element blocks in mesh order, so reading it back reproduces the node,
    boundary-edge and cell orders of ``m``."""
    names = list(m["names"])
    npatch = len(names)
    x, y = m["x"], m["y"]
    cells = m["cells"]
    bedges, bpatch = m["bedges"], m["bpatch"]
    nn = len(x)
    out = ["$MeshFormat", "4.1 0 8", "$EndMeshFormat", "$PhysicalNames", str(npatch + 1)]
    for p, nm in enumerate(names):
        out.append('1 %d "%s"' % (p + 1, nm))
    out.append('2 %d "internal"' % (npatch + 1))
    out += ["$EndPhysicalNames", "$Entities", "0 %d 1 0" % npatch]
    for p in range(npatch):
        out.append("%d 0 0 0 0 0 0 1 %d 0 " % (p + 1, p + 1))
    out.append("1 0 0 0 0 0 0 1 %d 0 " % (npatch + 1))
    out += ["$EndEntities", "$Nodes", "1 %d 1 %d" % (nn, nn), "2 1 0 %d" % nn]
    out += [str(i + 1) for i in range(nn)]
    out += ["%r %r 0" % (float(a), float(b)) for a, b in zip(x, y)]
    out.append("$EndNodes")
    # element blocks: boundary runs (consecutive edges of one patch), then cell runs of one type
    blocks = []
    start = 0
    B = len(bedges)
    while start < B:
        end = start
        while end < B and bpatch[end] == bpatch[start]:
            end += 1
        blocks.append(("b", int(bpatch[start]), start, end))
        start = end
    tri = cells[:, 3] < 0
    start = 0
    N = len(cells)
    while start < N:
        end = start
        while end < N and tri[end] == tri[start]:
            end += 1
        blocks.append(("c", bool(tri[start]), start, end))
        start = end
    total = B + N
    out += ["$Elements", "%d %d 1 %d" % (len(blocks), total, total)]
    eid = 1
    for kind, key, s, e in blocks:
        if kind == "b":
            out.append("1 %d 1 %d" % (key + 1, e - s))
            for k in range(s, e):
                out.append("%d %d %d " % (eid, bedges[k, 0] + 1, bedges[k, 1] + 1))
                eid += 1
        else:
            out.append("2 1 %d %d" % (2 if key else 3, e - s))
            for k in range(s, e):
                c = cells[k]
                if key:
                    out.append("%d %d %d %d " % (eid, c[0] + 1, c[1] + 1, c[2] + 1))
                else:
                    out.append("%d %d %d %d %d " % (eid, c[0] + 1, c[1] + 1, c[2] + 1, c[3] + 1))
                eid += 1
    out.append("$EndElements")
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")


def polar_sweep_cases(n_cases=256, seed=4, n_min=5000, n_max=200000, split=False):
    """Batched polar-sweep workload: ``n_cases`` NACA 4-digit airfoils with
    max camber m ~ U[0, 6]%, thickness t ~ U[8, 18]% and camber position
    p ~ U[0.2, 0.6]; cell count log-uniform in [n_min, n_max] (O-meshes with
    n_surf : n_rad = 2 : 1); angle of attack ~ U[-4, 12] degrees and Mach
    ~ U[0.1, 0.7].  Returns a list of dicts with the mesh and the flow."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n_cases):
        m = rng.uniform(0.0, 0.06)
        t = rng.uniform(0.08, 0.18)
        p = rng.uniform(0.2, 0.6)
        n = math.exp(rng.uniform(math.log(n_min), math.log(n_max)))
        aoa = rng.uniform(-4.0, 12.0)
        mach = rng.uniform(0.1, 0.7)
        n_rad = max(8, int(round(math.sqrt(n / (4.0 if split else 2.0)))))
        n_surf = 2 * n_rad
        mesh = airfoil_omesh(n_surf=n_surf, n_rad=n_rad, m=m, p=p, t=t, split=split, fade=2)
        out.append(dict(mesh=mesh, m=m, t=t, p=p, aoa_deg=aoa, mach=mach, n_cells=len(mesh["cells"])))
    return out


def _inside_polygon(px, py, vx, vy):
    """Even-odd test of points (px, py) against the closed polygon (vx, vy)."""
    inside = np.zeros(px.shape, bool)
    n = len(vx)
    for i in range(n):
        x0, y0, x1, y1 = vx[i], vy[i], vx[(i + 1) % n], vy[(i + 1) % n]
        crosses = (y0 > py) != (y1 > py)
        with np.errstate(divide="ignore", invalid="ignore"):
            xi = x0 + (py - y0) * (x1 - x0) / (y1 - y0)
        inside ^= crosses & (px < xi)
    return inside


def hybrid_airfoil(n_surf=512, bl_layers=60, first=1e-6, growth=1.1, r_far=100.0, fill_cells=170000, t=0.12,
                   seed=2, shuffle_seed=2):
    """Hybrid RANS mesh around a NACA 4-digit airfoil of chord 1: a
    structured boundary layer of ``bl_layers`` quad layers (first height
    ``first`` chords, geometric ``growth``) on ``n_surf`` cosine-spaced
    surface nodes, inside an unstructured triangular fill out to a circular
    far field of radius ``r_far`` chords centred at mid-chord.

    The fill is the Delaunay triangulation of the boundary layer's outer
    ring and of rings of points between it and the far-field circle (ring
    spacing growing geometrically, point counts decreasing outward so the
    triangles stay close to isotropic, tangential jitter from ``seed``),
    with the triangles inside the boundary layer removed; the ring growth is
    chosen so the fill has about ``fill_cells`` triangles.  Cells are
    shuffled with ``shuffle_seed``.  Patches: "wall" and "farfield"."""
    from scipy.spatial import Delaunay

    sx, sy = naca4_surface(n_surf, 0.0, 0.4, t)
    tx = np.roll(sx, -1) - np.roll(sx, 1)
    ty = np.roll(sy, -1) - np.roll(sy, 1)
    tn = np.sqrt(tx * tx + ty * ty)
    nx_, ny_ = ty / tn, -tx / tn
    h = first * (_pow(growth, np.arange(bl_layers + 1)) - 1.0) / (growth - 1.0)
    BX = sx[None, :] + h[:, None] * nx_[None, :]
    BY = sy[None, :] + h[:, None] * ny_[None, :]
    H, last = h[-1], h[-1] - h[-2]
    ex, ey = BX[-1], BY[-1]  # outer ring of the boundary layer
    ang0 = np.fromiter((math.atan2(a, b) for a, b in zip(ey.tolist(), (ex - 0.5).tolist())), np.float64)
    n_far = 128

    def rings(ratio):
        """Fill rings at distance d from the layer's edge, blended from the
        normal offset to the far-field circle, then the far-field ring."""
        rng = np.random.default_rng(seed)
        pts, d, step = [], 0.0, last * growth
        while True:
            d += step
            s = min(d / r_far, 1.0)
            if s >= 1.0:
                break
            per = 2 * np.pi * (0.5 + s * r_far)
            n_k = int(min(n_surf, max(32, round(per / step))))
            if n_k == n_surf:
                px = (1 - s) * (ex + d * nx_) + s * (0.5 + r_far * _cos(ang0))
                py = (1 - s) * (ey + d * ny_) + s * (r_far * _sin(ang0))
            else:
                a = ang0[0] + 2 * np.pi * (np.arange(n_k) + rng.uniform(-0.25, 0.25, n_k)) / n_k
                rad = np.interp(np.mod(a - ang0[0], 2 * np.pi), np.mod(ang0 - ang0[0], 2 * np.pi),
                                np.sqrt((ex - 0.5) * (ex - 0.5) + ey * ey), period=2 * np.pi)
                px = 0.5 + ((1 - s) * (rad + d) + s * r_far) * _cos(a)
                py = ((1 - s) * (rad + d) + s * r_far) * _sin(a)
            pts.append((px, py))
            step *= ratio
        a = 2 * np.pi * np.arange(n_far) / n_far
        pts.append((0.5 + r_far * _cos(a), r_far * _sin(a)))
        return pts

    lo, hi = 1.005, 1.5
    for _ in range(40):  # ring growth ratio for the requested fill size (points ~ triangles / 2)
        mid = 0.5 * (lo + hi)
        n_pts = sum(len(p[0]) for p in rings(mid))
        lo, hi = (mid, hi) if n_pts > fill_cells / 2 else (lo, mid)
    rr = rings(0.5 * (lo + hi))
    fx = np.concatenate([ex] + [p[0] for p in rr])
    fy = np.concatenate([ey] + [p[1] for p in rr])
    tri = Delaunay(np.stack([fx, fy], -1)).simplices
    keep = ~_inside_polygon(fx[tri].mean(1), fy[tri].mean(1), ex, ey)
    tri = tri[keep]
    # every edge of the layer's outer ring and of the far-field circle must be
    # an edge of exactly one kept triangle (a conforming mesh)
    e = np.sort(np.concatenate([tri[:, [0, 1]], tri[:, [1, 2]], tri[:, [2, 0]]]), 1)
    key = e[:, 0].astype(np.int64) * len(fx) + e[:, 1]
    uniq, cnt = np.unique(key, return_counts=True)
    cmap = dict(zip(uniq.tolist(), cnt.tolist()))
    j = np.arange(n_surf)
    ring_e = np.sort(np.stack([j, (j + 1) % n_surf], -1), 1)
    far0 = len(fx) - n_far
    k = np.arange(n_far)
    far_e = np.sort(np.stack([far0 + k, far0 + (k + 1) % n_far], -1), 1)
    for name, edges in (("boundary-layer edge", ring_e), ("far field", far_e)):
        bad = [tuple(x) for x in edges if cmap.get(int(x[0]) * len(fx) + int(x[1]), 0) != 1]
        if bad:
            raise RuntimeError("hybrid_airfoil: %d %s edges not recovered by the triangulation" % (len(bad), name))
    # assemble: boundary-layer nodes (ring-major), then the fill's own nodes
    nbl = (bl_layers + 1) * n_surf
    fill_map = np.concatenate([bl_layers * n_surf + j, nbl + np.arange(len(fx) - n_surf)])
    x = np.concatenate([BX.reshape(-1), fx[n_surf:]])
    y = np.concatenate([BY.reshape(-1), fy[n_surf:]])
    kk, jj = np.meshgrid(np.arange(bl_layers), np.arange(n_surf), indexing="ij")
    a = kk * n_surf + jj
    b = kk * n_surf + (jj + 1) % n_surf
    c = (kk + 1) * n_surf + (jj + 1) % n_surf
    d = (kk + 1) * n_surf + jj
    quads = np.stack([a, b, c, d], -1).reshape(-1, 4)
    tris = np.concatenate([fill_map[tri], np.full((len(tri), 1), -1)], 1)
    cells = np.concatenate([quads, tris]).astype(np.int32)
    if shuffle_seed is not None:
        cells = cells[np.random.default_rng(shuffle_seed).permutation(len(cells))]
    wall = np.stack([j, (j + 1) % n_surf], -1)
    far = np.stack([fill_map[far0 + k], fill_map[far0 + (k + 1) % n_far]], -1)
    bedges = np.concatenate([wall, far]).astype(np.int32)
    bpatch = np.concatenate([np.zeros(n_surf), np.ones(n_far)]).astype(np.int32)
    return dict(x=x, y=y, cells=cells, bedges=bedges, bpatch=bpatch, names=["wall", "farfield"],
                n_bl_quads=len(quads), n_fill_triangles=len(tri), bl_thickness=H)
