"""Lattices in the reference's file layout, built from geometry.

A lattice is what the reference's solver reads from its Node and BC files
(Source code/lbm-solver_final/FilesReading.cu:270-347): a fluid/solid flag per
node (x fastest) and a list of boundary links (i, j, k, dir, type, id), where
`dir` is the lattice direction from a fluid node into the boundary and `type`
is 1 wall, 2 inlet, 3 outlet, 4 periodic, 5 symmetry.

Builders here emit the workloads this engine is measured on:

* cavity2d / cavity3d -- lid-driven cavities: every node fluid, a link for each
  direction leaving the domain, inlet-typed where it leaves through the lid.
* sphere_duct -- a duct packed with non-overlapping spheres of random radii
  until a target porosity, pressure faces at both ends of the long axis.
* channel2d -- a 2D channel with circular and rectangular obstacles.
* cylinder_channel2d / sphere_cavity3d -- curved-wall cases: every link into
  the cylinder or sphere is a wall link with its exact fraction q (link_q).
"""
from dataclasses import dataclass, field

import numpy as np

# Reference direction order (GpuInit.cu:97-98, :835-837).
CX2 = np.array([0, 1, 0, -1, 0, 1, -1, -1, 1])
CY2 = np.array([0, 0, 1, 0, -1, 1, 1, -1, -1])
CX3 = np.array([0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0])
CY3 = np.array([0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1])
CZ3 = np.array([0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1])
W2 = np.array([4 / 9] + [1 / 9] * 4 + [1 / 36] * 4)
W3 = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)


@dataclass
class Lattice:
    dims: int
    n: int
    m: int
    h: int
    node_type: np.ndarray                      # int32, n*m*h, x fastest
    bc: np.ndarray = field(default=None)       # int32 (num_conns, 6): i, j, k, dir, type, id

    def __post_init__(self):
        self.node_type = np.ascontiguousarray(self.node_type.reshape(-1), dtype=np.int32)
        if self.bc is None:
            self.bc = np.zeros((0, 6), np.int32)
        self.bc = np.ascontiguousarray(self.bc, dtype=np.int32)

    @property
    def q(self):
        return 9 if self.dims == 2 else 19

    @property
    def num_nodes(self):
        return self.n * self.m * self.h

    @property
    def num_fluid(self):
        return int(self.node_type.sum())

    def coords(self, delta=None):
        """Node coordinates as the generator writes them: index * spacing."""
        d = delta if delta is not None else 1.0 / max(self.n - 1, 1)
        idx = np.arange(self.num_nodes)
        x = (idx % self.n) * d
        y = ((idx // self.n) % self.m) * d
        z = (idx // (self.n * self.m)) * d
        return x, y, z


def _boundary_links(dims, n, m, h, fluid, face_type):
    """Links of fluid nodes whose direction leaves the domain.

    face_type(axis, side) -> BC type for a link leaving through that face, or
    0 for none.  A link leaving through several faces takes the first non-zero
    type in the order x-, x+, y-, y+, z-, z+.
    """
    if dims == 2:
        cxs, cys, czs = CX2, CY2, np.zeros(9, int)
    else:
        cxs, cys, czs = CX3, CY3, CZ3
    q = len(cxs)
    idx = np.nonzero(fluid)[0]
    x = idx % n
    y = (idx // n) % m
    z = idx // (n * m)
    on_edge = (x == 0) | (x == n - 1) | (y == 0) | (y == m - 1)
    if dims == 3:
        on_edge |= (z == 0) | (z == h - 1)
    idx, x, y, z = idx[on_edge], x[on_edge], y[on_edge], z[on_edge]
    out = []
    for d in range(1, q):
        tx, ty, tz = x + cxs[d], y + cys[d], z + czs[d]
        t = np.zeros(idx.shape, np.int32)
        for axis, coord, size in ((0, tx, n), (1, ty, m), (2, tz, h)):
            for side, sel in ((0, coord < 0), (1, coord > size - 1)):
                ft = face_type(axis, side)
                if ft:
                    t = np.where((t == 0) & sel, ft, t)
        leave = (tx < 0) | (tx > n - 1) | (ty < 0) | (ty > m - 1) | (tz < 0) | (tz > h - 1)
        sel = leave & (t > 0)
        if sel.any():
            k = np.count_nonzero(sel)
            out.append(np.stack([x[sel], y[sel], z[sel], np.full(k, d), t[sel], np.zeros(k, int)], 1))
    if not out:
        return np.zeros((0, 6), np.int32)
    bc = np.concatenate(out).astype(np.int32)
    # node-major order, as a generator sweeping the lattice would write them
    order = np.lexsort((bc[:, 3], bc[:, 0] + n * (bc[:, 1] + m * bc[:, 2])))
    return bc[order]


def cavity2d(n, m=None):
    """Lid-driven cavity: all nodes fluid, walls on three sides, the lid
    (links leaving through y = m-1) an inlet."""
    m = n if m is None else m
    fluid = np.ones(n * m, np.int32)

    def ft(axis, side):
        return 2 if (axis == 1 and side == 1) else 1
    return Lattice(2, n, m, 1, fluid, _boundary_links(2, n, m, 1, fluid, ft))


def cavity3d(n, m=None, h=None):
    """3D lid-driven cavity with the lid at z = h-1."""
    m = n if m is None else m
    h = n if h is None else h
    fluid = np.ones(n * m * h, np.int32)

    def ft(axis, side):
        return 2 if (axis == 2 and side == 1) else 1
    return Lattice(3, n, m, h, fluid, _boundary_links(3, n, m, h, fluid, ft))


def periodic_channel3d(n, m=None, h=None, periodic_axes=(0,)):
    """Lid-driven channel in the reference's BC types: links leaving through
    the faces of `periodic_axes` are periodic (type 4), the lid z = h-1 an
    inlet, every other face a wall."""
    m = n if m is None else m
    h = n if h is None else h
    fluid = np.ones(n * m * h, np.int32)

    def ft(axis, side):
        if axis in periodic_axes:
            return 4
        return 2 if (axis == 2 and side == 1) else 1
    return Lattice(3, n, m, h, fluid, _boundary_links(3, n, m, h, fluid, ft))


class SplitMix64:
    """SplitMix64 (Steele, Lea and Flood, OOPSLA 2014) with uniform doubles
    from the top 53 bits.  The library's emitters (lattice_emit.cpp) draw the
    same sequence, so a builder here and the Node/BC files emitted there give
    the same lattice for a seed."""
    MASK = (1 << 64) - 1

    def __init__(self, seed):
        self.s = int(seed) & self.MASK

    def next(self):
        self.s = (self.s + 0x9E3779B97F4A7C15) & self.MASK
        z = self.s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & self.MASK
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & self.MASK
        return z ^ (z >> 31)

    def uniform(self, lo=0.0, hi=1.0):
        return lo + (hi - lo) * ((self.next() >> 11) * 2.0 ** -53)


def pack_spheres(shape, porosity=0.70, rmin=6.0, rmax=14.0, seed=0, margin_axis=2, margin=2,
                 max_attempts=2_000_000):
    """Random sequential insertion of non-overlapping spheres.

    Radii uniform in [rmin, rmax], centres uniform in the box (kept `margin`
    nodes plus a radius away from both ends of `margin_axis`, so the pressure
    faces stay fluid); spheres are added until the solid fraction reaches
    1 - porosity.  Per attempt the draws are r, x, y, z, then the margin
    axis' coordinate again within its band (lbm_pack_spheres makes the same
    draws and tests in the same order).  Returns (solid mask (z, y, x) bool,
    spheres (k, 4)).
    """
    n, m, h = shape
    rng = SplitMix64(seed)
    target = (1.0 - porosity) * n * m * h
    ext = [float(n - 1), float(m - 1), float(h - 1)]
    solid = np.zeros((h, m, n), bool)
    cxs, cys, czs, rads = (np.zeros(0) for _ in range(4))
    solid_count = 0
    attempts = 0
    while solid_count < target and attempts < max_attempts:
        attempts += 1
        r = rng.uniform(rmin, rmax)
        c = [rng.uniform() * ext[0], rng.uniform() * ext[1], rng.uniform() * ext[2]]
        lo = margin + r
        hi = ext[margin_axis] - margin - r
        c[margin_axis] = lo + rng.uniform() * max(hi - lo, 0.0)
        if rads.size:
            dx, dy, dz = cxs - c[0], cys - c[1], czs - c[2]
            rr = rads + r
            if np.any(dx * dx + dy * dy + dz * dz < rr * rr):
                continue
        cxs, cys, czs, rads = (np.append(a, v) for a, v in ((cxs, c[0]), (cys, c[1]), (czs, c[2]), (rads, r)))
        x0, y0, z0 = c
        xs = slice(max(int(np.floor(x0 - r)), 0), min(int(np.ceil(x0 + r)) + 1, n))
        ys = slice(max(int(np.floor(y0 - r)), 0), min(int(np.ceil(y0 + r)) + 1, m))
        zs = slice(max(int(np.floor(z0 - r)), 0), min(int(np.ceil(z0 + r)) + 1, h))
        zz, yy, xx = np.meshgrid(np.arange(zs.start, zs.stop, dtype=np.float64),
                                 np.arange(ys.start, ys.stop, dtype=np.float64),
                                 np.arange(xs.start, xs.stop, dtype=np.float64), indexing="ij")
        ddx, ddy, ddz = xx - x0, yy - y0, zz - z0
        inside = ddx * ddx + ddy * ddy + ddz * ddz <= r * r
        sub = solid[zs, ys, xs]
        solid_count += int(np.count_nonzero(inside & ~sub))
        sub |= inside
    spheres = np.stack([cxs, cys, czs, rads], 1) if rads.size else np.zeros((0, 4))
    return solid, spheres


def sphere_duct(n=256, m=256, h=512, porosity=0.70, rmin=6.0, rmax=14.0, seed=0):
    """Pressure-driven duct along z packed with spheres: inlet face z = 0,
    outlet face z = h-1, the four side faces and the spheres are walls (in
    physics mode, links into solid or out of the domain bounce back, so only
    the two pressure faces need BC links)."""
    solid, spheres = pack_spheres((n, m, h), porosity, rmin, rmax, seed, margin_axis=2)
    fluid = (~solid).astype(np.int32).reshape(-1)

    def ft(axis, side):
        if axis == 2:
            return 2 if side == 0 else 3
        return 0
    lat = Lattice(3, n, m, h, fluid, _boundary_links(3, n, m, h, fluid, ft))
    lat.spheres = spheres
    return lat


def channel2d(n=1024, m=256, seed=0, n_obstacles=None, size_scale=1.0):
    """2D channel along x with 1-6 circles (radius 8-32) and rectangles
    (sides 10-60), non-overlapping and clear of the inlet and outlet; walls at
    y = 0 and y = m-1, inlet x = 0, outlet x = n-1.  size_scale multiplies the
    obstacle sizes (0.25 for a 256 x 64 channel with the proportions of the
    1024 x 256 one).  Draws from SplitMix64(seed) in the order
    lbm_emit_channel2d makes them."""
    rng = SplitMix64(seed)
    k = n_obstacles if n_obstacles is not None else 1 + min(int(rng.uniform() * 6.0), 5)
    solid = np.zeros((m, n), bool)
    boxes = []
    yy, xx = np.mgrid[0:m, 0:n].astype(np.float64)
    placed = 0
    tries = 0
    s = float(size_scale)
    while placed < k and tries < 10_000:
        tries += 1
        rmax = min(32.0 * s, (m - 8) / 2.0, n * 0.3)
        smax = min(60.0 * s, m - 8.0, n * 0.5)
        if rng.uniform() < 0.5:
            r = rng.uniform(min(8.0 * s, rmax), rmax)
            cx = rng.uniform(n * 0.1 + r, n * 0.85 - r)
            cy = rng.uniform(r + 3, m - 4 - r)
            bb = (cx - r, cy - r, cx + r, cy + r)
            shape = ("circle", cx, cy, r)
        else:
            w = rng.uniform(min(10.0 * s, smax), smax)
            hh = rng.uniform(min(10.0 * s, smax), smax)
            x0 = rng.uniform(n * 0.1, n * 0.85 - w)
            y0 = rng.uniform(3, m - 4 - hh)
            bb = (x0, y0, x0 + w, y0 + hh)
            shape = ("rect", x0, y0, w, hh)
        if any(not (bb[2] + 2 < b[0] or b[2] + 2 < bb[0] or bb[3] + 2 < b[1] or b[3] + 2 < bb[1]) for b in boxes):
            continue
        boxes.append(bb)
        if shape[0] == "circle":
            dx, dy = xx - shape[1], yy - shape[2]
            solid |= dx * dx + dy * dy <= shape[3] * shape[3]
        else:
            solid |= (xx >= shape[1]) & (xx <= shape[1] + shape[3]) & (yy >= shape[2]) & (yy <= shape[2] + shape[4])
        placed += 1
    fluid = (~solid).astype(np.int32).reshape(-1)

    def ft(axis, side):
        if axis == 0:
            return 2 if side == 0 else 3
        return 1
    return Lattice(2, n, m, 1, fluid, _boundary_links(2, n, m, 1, fluid, ft))


def _curved_links(dims, n, m, h, fluid, solid_of, centre, radius, outer, outer_q):
    """Wall links of fluid nodes into a ball (disk in 2D) with their exact
    fractions q along the link (the smaller root of |x + t c - centre| = r),
    merged with the domain-leaving links `outer` (fraction outer_q), in
    node-major, direction order.  Returns (bc, link_q).

    A q < 1/2 link reads the upstream population at the flat index
    node + dir N + c(dir) of the direction-major array (the reference's
    addressing); an outer wall link for which that index falls past either
    end of the array, where the reference's read is undefined, takes 1/2."""
    if dims == 2:
        cxs, cys, czs = CX2, CY2, np.zeros(9, int)
    else:
        cxs, cys, czs = CX3, CY3, CZ3
    idx = np.nonzero(fluid)[0]
    x, y, z = idx % n, (idx // n) % m, idx // (n * m)
    rows, qs = [], []
    cen = np.asarray(centre, float)
    for d in range(1, len(cxs)):
        tx, ty, tz = x + cxs[d], y + cys[d], z + czs[d]
        inside = (tx >= 0) & (tx < n) & (ty >= 0) & (ty < m) & (tz >= 0) & (tz < h)
        sel = np.zeros(idx.shape, bool)
        sel[inside] = solid_of(tx[inside], ty[inside], tz[inside])
        if not sel.any():
            continue
        p = np.stack([x[sel], y[sel], z[sel]], 1).astype(float) - cen[: 3]
        c = np.array([cxs[d], cys[d], czs[d]], float)
        a = c @ c
        b = 2 * (p @ c)
        cc = (p * p).sum(1) - radius * radius
        t = (-b - np.sqrt(np.maximum(b * b - 4 * a * cc, 0))) / (2 * a)
        k = int(sel.sum())
        rows.append(np.stack([x[sel], y[sel], z[sel], np.full(k, d), np.ones(k, int), np.zeros(k, int)], 1))
        qs.append(np.clip(t, 0.0, 1.0))
    rows.append(outer)
    if outer.size:
        d = outer[:, 3]
        flat = (outer[:, 0] + n * (outer[:, 1] + m * outer[:, 2]) + d * (n * m * h)
                - (cxs[d] + n * cys[d] + n * m * czs[d]))
        inside = (flat >= 0) & (flat < len(cxs) * n * m * h)
        qs.append(np.where((outer[:, 4] == 1) & inside, outer_q, 0.5))
    else:
        qs.append(np.zeros(0))
    bc = np.concatenate(rows).astype(np.int32)
    q = np.concatenate(qs)
    order = np.lexsort((bc[:, 3], bc[:, 0] + n * (bc[:, 1] + m * bc[:, 2])))
    return bc[order], q[order]


def cylinder_channel2d(n=48, m=24, centre=None, radius=None, outer_q=0.5):
    """2D channel along x (inlet x = 0, outlet x = n-1, walls y = 0 and m-1)
    around a cylinder, with curved walls: every link of a fluid node into the
    cylinder is a wall link carrying its exact fraction q (lat.link_q, one
    per BC row), the outer walls' links carry outer_q."""
    cx, cy = centre if centre is not None else (0.35 * n, 0.5 * m - 0.37)
    r = radius if radius is not None else 0.21 * m
    yy, xx = np.mgrid[0:m, 0:n]
    solid = (xx - cx) ** 2 + (yy - cy) ** 2 <= r * r
    fluid = (~solid).astype(np.int32).reshape(-1)

    def ft(axis, side):
        if axis == 0:
            return 2 if side == 0 else 3
        return 1
    outer = _boundary_links(2, n, m, 1, fluid, ft)
    bc, q = _curved_links(2, n, m, 1, fluid, lambda tx, ty, tz: solid[ty, tx], (cx, cy, 0.0), r, outer, outer_q)
    lat = Lattice(2, n, m, 1, fluid, bc)
    lat.link_q = q
    return lat


def sphere_cavity3d(n=14, m=12, h=12, centre=None, radius=None, outer_q=0.5):
    """3D lid-driven cavity (lid z = h-1) around a sphere, with curved walls
    as in cylinder_channel2d (lat.link_q)."""
    c = centre if centre is not None else (0.45 * n + 0.13, 0.5 * m - 0.29, 0.45 * h + 0.21)
    r = radius if radius is not None else 0.24 * min(n, m, h)
    zz, yy, xx = np.mgrid[0:h, 0:m, 0:n]
    solid = (xx - c[0]) ** 2 + (yy - c[1]) ** 2 + (zz - c[2]) ** 2 <= r * r
    fluid = (~solid).astype(np.int32).reshape(-1)

    def ft(axis, side):
        return 2 if (axis == 2 and side == 1) else 1
    outer = _boundary_links(3, n, m, h, fluid, ft)
    bc, q = _curved_links(3, n, m, h, fluid, lambda tx, ty, tz: solid[tz, ty, tx], c, r, outer, outer_q)
    lat = Lattice(3, n, m, h, fluid, bc)
    lat.link_q = q
    return lat


def read_node_file(path, dims):
    """Node file (FilesReading.cu:270-305): `i j x y fluid` (2D, spaces) or
    `i<TAB>j<TAB>k<TAB>x<TAB>y<TAB>z<TAB>fluid` (3D).  Returns columns."""
    a = np.loadtxt(path, ndmin=2)
    return a


def read_bc_file(path, dims):
    """BC file (FilesReading.cu:307-347): `i j dir bc x y id` (2D) or
    `i j k dir bc x y z id` (3D)."""
    return np.loadtxt(path, ndmin=2)


def from_files(node_path, bc_path):
    """Build a Lattice from reference-format Node and BC files."""
    nodes = np.loadtxt(node_path, ndmin=2)
    dims = 3 if nodes.shape[1] == 7 else 2
    bcs = np.loadtxt(bc_path, ndmin=2)
    if dims == 3:
        n, m, h = int(nodes[-1, 0]) + 1, int(nodes[-1, 1]) + 1, int(nodes[-1, 2]) + 1
        fluid = nodes[:, 6]
        bc = np.stack([bcs[:, 0], bcs[:, 1], bcs[:, 2], bcs[:, 3], bcs[:, 4], bcs[:, 8]], 1)
    else:
        n, m, h = int(nodes[-1, 0]) + 1, int(nodes[-1, 1]) + 1, 1
        fluid = nodes[:, 4]
        bc = np.stack([bcs[:, 0], bcs[:, 1], np.zeros(len(bcs)), bcs[:, 2], bcs[:, 3], bcs[:, 6]], 1)
    return Lattice(dims, n, m, h, fluid.astype(np.int32), bc.astype(np.int32))


def from_files_native(node_path, bc_path):
    """Build a Lattice from reference-format Node and BC files with the
    library's readers (lbm_read_node_file, lbm_read_bc_file): the path a run
    takes, and fast enough for lattices of tens of millions of nodes."""
    import ctypes as C

    from . import native as N
    lib = N.lib()
    np_ = node_path.encode()
    bp = bc_path.encode()
    dims = int(lib.lbm_node_file_dims(np_))
    if dims not in (2, 3):
        raise ValueError("cannot tell the dimension of %s" % node_path)
    count = int(lib.lbm_count_lines(np_))
    nb = int(lib.lbm_count_lines(bp))
    ii, jj, kk, tt = (np.zeros(count, np.int32) for _ in range(4))
    xs = [np.zeros(count, np.float32) for _ in range(3)]
    ip = lambda a: a.ctypes.data_as(C.POINTER(C.c_int))  # noqa: E731
    fp = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))  # noqa: E731
    N.check(lib.lbm_read_node_file(np_, dims, count, ip(ii), ip(jj), ip(kk), fp(xs[0]), fp(xs[1]), fp(xs[2]),
                                   ip(tt)))
    n, m, h = int(ii.max()) + 1, int(jj.max()) + 1, (int(kk.max()) + 1 if dims == 3 else 1)
    node = ii.astype(np.int64) + n * (jj.astype(np.int64) + m * kk.astype(np.int64))
    fluid = np.zeros(n * m * h, np.int32)
    fluid[node] = tt
    cols = [np.zeros(nb, np.int32) for _ in range(6)]
    bx = [np.zeros(nb, np.float32) for _ in range(3)]
    if nb:
        N.check(lib.lbm_read_bc_file(bp, dims, nb, ip(cols[0]), ip(cols[1]), ip(cols[2]), ip(cols[3]), ip(cols[4]),
                                     fp(bx[0]), fp(bx[1]), fp(bx[2]), ip(cols[5])))
    if dims == 2:
        cols[2][:] = 0
    return Lattice(dims, n, m, h, fluid, np.stack(cols, 1))


def write_files(lat, node_path, bc_path, delta=None):
    """Write a Lattice as reference-format Node and BC files (the layout
    readNodeFile/readConnFile read, FilesReading.cu:270-347): 2D
    `i j x y fluid` and `i j dir type x y id`; 3D tab-separated
    `i j k x y z fluid` and `i j k<TAB><TAB>dir type x y z id`.  Coordinates
    are index * delta (default 1/(n-1)); a BC line's coordinates are those of
    its node."""
    x, y, z = lat.coords(delta)
    idx = np.arange(lat.num_nodes)
    i, j, k = idx % lat.n, (idx // lat.n) % lat.m, idx // (lat.n * lat.m)
    with open(node_path, "w") as f:
        if lat.dims == 2:
            for r in range(lat.num_nodes):
                f.write("%d %d %.6f %.6f %d\n" % (i[r], j[r], x[r], y[r], lat.node_type[r]))
        else:
            for r in range(lat.num_nodes):
                f.write("%d\t%d\t%d\t%.6f\t%.6f\t%.6f\t%d\n" % (i[r], j[r], k[r], x[r], y[r], z[r],
                                                                lat.node_type[r]))
    with open(bc_path, "w") as f:
        for bi, bj, bk, d, t, bid in lat.bc:
            r = bi + lat.n * (bj + lat.m * bk)
            if lat.dims == 2:
                f.write("%d %d %d %d %.6f %.6f %d\n" % (bi, bj, d, t, x[r], y[r], bid))
            else:
                f.write("%d\t%d\t%d\t\t%d\t%d\t%.6f\t%.6f\t%.6f\t%d\n" % (bi, bj, bk, d, t, x[r], y[r], z[r], bid))


def write_starcd(prefix, vertices, faces):
    """Write STAR-CD geometry in the generator's input layout: `<prefix>.vrt`
    lines `id x y z` and `<prefix>.bnd` lines `id p1 p2 p3 p4 bcid 0 TYPE`
    with TYPE one of WALL, INLE, OUTL, CYCL, SYMP (GeomRead.cpp:40-99)."""
    with open(prefix + ".vrt", "w") as f:
        for i, (x, y, z) in enumerate(vertices, 1):
            f.write("%9d      %+.9e%+.9e%+.9e\n" % (i, x, y, z))
    with open(prefix + ".bnd", "w") as f:
        for i, (pts, bcid, kind) in enumerate(faces, 1):
            f.write("%8d %14d %8d %8d %8d %6d %6d      %s\n" % (i, pts[0], pts[1], pts[2], pts[3], bcid, 0, kind))


def box_geometry(lo, hi, kinds, first_vertex=1, first_bcid=1):
    """Vertices and faces of an axis-aligned box.  kinds: dict face -> TYPE
    for faces 'x-','x+','y-','y+','z-','z+'."""
    (x0, y0, z0), (x1, y1, z1) = lo, hi
    v = [(x0, y0, z0), (x1, y0, z0), (x1, y1, z0), (x0, y1, z0),
         (x0, y0, z1), (x1, y0, z1), (x1, y1, z1), (x0, y1, z1)]
    b = first_vertex
    quads = {"z-": (0, 1, 2, 3), "z+": (4, 5, 6, 7), "y-": (0, 1, 5, 4),
             "y+": (3, 2, 6, 7), "x-": (0, 3, 7, 4), "x+": (1, 2, 6, 5)}
    faces = []
    for k, name in enumerate(("x-", "x+", "y-", "y+", "z-", "z+")):
        q = quads[name]
        faces.append(((b + q[0], b + q[1], b + q[2], b + q[3]), first_bcid + k, kinds.get(name, "WALL")))
    return v, faces


def generate(vrt, bnd, n, seed, complexity=1, out_prefix="lattice"):
    """Run the library's lattice generator (bit-identical to the reference
    latticegen); returns (node path, bc path, (n, m, h))."""
    import ctypes as C
    from . import native as N
    L = N.lib()
    fn = L.lbm_latticegen
    fn.restype = C.c_int
    fn.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.c_double, C.c_double, C.c_double, C.c_int,
                   C.c_char_p, C.c_char_p, C.POINTER(C.c_int)]
    dims = (C.c_int * 3)()
    node, bc = out_prefix + "_Node.dat", out_prefix + "_BC.dat"
    rc = fn(vrt.encode(), bnd.encode(), int(n), float(seed[0]), float(seed[1]), float(seed[2]),
            int(complexity), node.encode(), bc.encode(), dims)
    if rc != 0:
        L.lbm_latticegen_error.restype = C.c_char_p
        raise N.LbmError(rc, L.lbm_latticegen_error().decode())
    return node, bc, tuple(dims)
