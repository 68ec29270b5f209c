"""Procedural tetrahedral pipe meshes: the synthetic input of the fluid/FSI hot path.

The reference reads its meshes from VTU files (``read_msh.cpp``); those files are not
available, so the pipe is built in code.  Construction:

* cross-section: an O-grid of quads (``nc x nc`` square core plus four ring blocks of
  ``nc x nr`` quads reaching the circular wall), each quad cut into two triangles;
* axial extrusion into ``nz`` layers of triangular prisms;
* each prism is split into three tets with the minimum-global-index rule (the face
  diagonal of every quad side goes through its smallest node id), which makes the
  tet mesh conforming without any neighbour bookkeeping;
* tets are oriented so that the TET4 Jacobian of ``nn.cpp:gnn`` (``nn.cpp:512``)
  is positive: the reference multiplies the quadrature weight by ``Jac`` unsigned
  (``fluid.cpp:627``).

Optional seeded wall perturbation r(theta, z) = R (1 + sum_k a_k sin(m_k theta +
2 pi n_k z / L + phi_k)); every node radius is scaled by r/R (affine in the radius).

Face sets follow the reference's ``faceType`` (``ComMod.h:520``): triangle
connectivity, the id of the tet owning each triangle (``gE``) and the sorted node
list (``gN``).
"""
from __future__ import annotations

import dataclasses
import numpy as np


@dataclasses.dataclass
class Face:
    name: str
    ien: np.ndarray   # (nFaEl, 3) int32 global node ids
    gE: np.ndarray    # (nFaEl,) int32 owning tet id
    gN: np.ndarray    # (nFaNo,) int32 sorted unique node ids


@dataclasses.dataclass
class PipeMesh:
    x: np.ndarray         # (nNo, 3) float64 coordinates
    ien: np.ndarray       # (nEl, 4) int32 tet connectivity
    faces: dict           # name -> Face ('inlet', 'outlet', 'wall')
    radius: float
    length: float
    inlet_profile: np.ndarray  # (nNo_inlet,) parabolic profile 1 - r^2/Rwall^2 at inlet.gN
    params: dict
    # FSI pipes only: element domains (mshType eId: bit 0 fluid, bit 1 solid)
    eid: np.ndarray | None = None

    @property
    def nNo(self) -> int:
        return int(self.x.shape[0])

    @property
    def nEl(self) -> int:
        return int(self.ien.shape[0])


def _cross_section(nc: int, nr: int, radius: float, core_frac: float = 0.55, nrs: int = 0,
                   thickness: float = 0.0):
    """O-grid quads of the unit-radius disc scaled by ``radius``, optionally followed by
    ``nrs`` rings of quads of a wall annulus from ``radius`` to ``radius + thickness``.

    Returns node xy (nN, 2), quads (nQ, 4) counter-clockwise, the ids of the nodes on
    the circle of radius ``radius`` (in angular order) and on the outermost circle."""
    a = core_frac * radius / np.sqrt(2.0)
    # core square nodes (nc+1)^2
    t = np.linspace(-a, a, nc + 1)
    X, Y = np.meshgrid(t, t, indexing="ij")
    core = np.stack([X.ravel(), Y.ravel()], axis=1)

    def cid(i, j):
        return i * (nc + 1) + j

    quads = []
    for i in range(nc):
        for j in range(nc):
            quads.append((cid(i, j), cid(i + 1, j), cid(i + 1, j + 1), cid(i, j + 1)))

    # boundary loop of the core square, counter-clockwise, 4*nc nodes
    loop = []
    for i in range(nc):
        loop.append(cid(i, 0))           # bottom edge, left->right
    for j in range(nc):
        loop.append(cid(nc, j))          # right edge, bottom->top
    for i in range(nc, 0, -1):
        loop.append(cid(i, nc))          # top edge, right->left
    for j in range(nc, 0, -1):
        loop.append(cid(0, j))           # left edge, top->bottom
    loop = np.asarray(loop)
    nloop = loop.size

    ps = core[loop]
    ang = np.arctan2(ps[:, 1], ps[:, 0])
    pc = radius * np.stack([np.cos(ang), np.sin(ang)], axis=1)

    nodes = [core]
    ring_ids = [loop]
    base = core.shape[0]
    for j in range(1, nr + 1):
        s = j / nr
        # grade towards the wall a little so the boundary layer is resolved
        s = 1.0 - (1.0 - s) ** 1.3
        nodes.append(ps + s * (pc - ps))
        ring_ids.append(base + np.arange(nloop))
        base += nloop
    unit = np.stack([np.cos(ang), np.sin(ang)], axis=1)
    for j in range(1, nrs + 1):
        nodes.append((radius + thickness * j / nrs) * unit)
        ring_ids.append(base + np.arange(nloop))
        base += nloop
    xy = np.concatenate(nodes, axis=0)
    for j in range(nr + nrs):
        inner, outer = ring_ids[j], ring_ids[j + 1]
        for k in range(nloop):
            k1 = (k + 1) % nloop
            quads.append((inner[k], inner[k1], outer[k1], outer[k]))
    return xy, np.asarray(quads, dtype=np.int64), ring_ids[nr], ring_ids[-1]


def _split_prisms(bot: np.ndarray, top: np.ndarray) -> np.ndarray:
    """Split prisms (bot[i] = v0,v1,v2 ; top[i] = v3,v4,v5 above them) into 3 tets each.

    Minimum-global-index rule: rotate/reflect each prism so that its smallest node is
    v0, then cut the quad opposite to v0 through the smaller of its two diagonals'
    minimum nodes.  Every quad face is thereby cut through its smallest node, which
    is what neighbouring prisms agree on."""
    P = np.concatenate([bot, top], axis=1)  # (n, 6)
    n = P.shape[0]
    # the 6 symmetries of a prism that keep its structure: 3 rotations x optional reflection
    perms = np.array([
        [0, 1, 2, 3, 4, 5], [1, 2, 0, 4, 5, 3], [2, 0, 1, 5, 3, 4],
        [3, 5, 4, 0, 2, 1], [4, 3, 5, 1, 0, 2], [5, 4, 3, 2, 1, 0],
    ])
    amin = np.argmin(P, axis=1)
    # perm index whose first entry equals amin
    first = perms[:, 0]
    pidx = np.argmax(first[None, :] == amin[:, None], axis=1)
    Q = np.take_along_axis(P, perms[pidx], axis=1)
    v0, v1, v2, v3, v4, v5 = (Q[:, i] for i in range(6))
    c = np.minimum(v1, v5) < np.minimum(v2, v4)
    t1 = np.where(c[:, None], np.stack([v0, v1, v2, v5], 1), np.stack([v0, v1, v2, v4], 1))
    t2 = np.where(c[:, None], np.stack([v0, v1, v5, v4], 1), np.stack([v0, v4, v2, v5], 1))
    t3 = np.stack([v0, v4, v5, v3], 1)
    return np.stack([t1, t2, t3], axis=1).reshape(3 * n, 4)


def _orient(x: np.ndarray, ien: np.ndarray) -> np.ndarray:
    """Swap two nodes of every tet whose TET4 Jacobian det[x1-x4, x2-x4, x3-x4] < 0."""
    x4 = x[ien[:, 3]]
    d1 = x[ien[:, 0]] - x4
    d2 = x[ien[:, 1]] - x4
    d3 = x[ien[:, 2]] - x4
    det = np.einsum("ij,ij->i", d1, np.cross(d2, d3))
    neg = det < 0
    ien = ien.copy()
    ien[neg, 0], ien[neg, 1] = ien[neg, 1].copy(), ien[neg, 0].copy()
    return ien


def _match_faces(tri: np.ndarray, ien: np.ndarray, cand: np.ndarray, nNo: int) -> np.ndarray:
    """For each boundary triangle, the id of the candidate tet that owns it."""
    def key(a):
        s = np.sort(a, axis=1).astype(np.int64)
        return (s[:, 0] * nNo + s[:, 1]) * nNo + s[:, 2]
    faces_local = np.array([[0, 1, 2], [0, 1, 3], [0, 2, 3], [1, 2, 3]])
    T = ien[cand]
    fk = np.concatenate([key(T[:, f]) for f in faces_local])
    fe = np.concatenate([cand for _ in range(4)])
    order = np.argsort(fk)
    fk, fe = fk[order], fe[order]
    tk = key(tri)
    pos = np.searchsorted(fk, tk)
    if np.any(pos >= fk.size) or np.any(fk[np.minimum(pos, fk.size - 1)] != tk):
        raise RuntimeError("boundary triangle without an owning tet")
    return fe[pos].astype(np.int32)


def make_pipe(nc: int, nr: int, nz: int, radius: float = 0.5, length: float = 5.0,
              perturb_modes: int = 0, seed: int = 20261203, max_amp: float = 0.1,
              nrs: int = 0, thickness: float = 0.1) -> PipeMesh:
    """Build the tet pipe.  Nodes are numbered layer by layer (z outer), which keeps
    the CSR bandwidth of the block matrix near one cross-section.

    With ``nrs > 0`` the pipe gets a solid wall annulus of ``nrs`` element rings from
    ``radius`` to ``radius + thickness`` that shares its inner surface nodes with the
    lumen (the monolithic FSI set-up of the reference's fsi/pipe_3d case):
    ``eid`` marks fluid (1) and solid (2) elements, the faces 'inlet'/'outlet' are the
    lumen's, 'wall' is the fluid-solid interface (owner: the fluid tet), and
    'wall_inlet', 'wall_outlet', 'wall_outer' bound the solid."""
    xy, quads, wall_loop, outer_loop = _cross_section(nc, nr, radius, nrs=nrs, thickness=thickness)
    nxy = xy.shape[0]
    z = np.linspace(0.0, length, nz + 1)
    x = np.empty(((nz + 1) * nxy, 3))
    for k in range(nz + 1):
        x[k * nxy:(k + 1) * nxy, 0:2] = xy
        x[k * nxy:(k + 1) * nxy, 2] = z[k]

    params = dict(nc=nc, nr=nr, nz=nz, radius=radius, length=length, seed=seed,
                  perturb_modes=perturb_modes)
    rwall_ratio = np.ones(x.shape[0])
    if perturb_modes > 0:
        rng = np.random.default_rng(seed)
        amp = rng.uniform(0.0, max_amp / (perturb_modes * 1.0), perturb_modes)
        m = rng.integers(1, 7, perturb_modes)
        nk = rng.integers(1, 4, perturb_modes)
        phi = rng.uniform(0.0, 2.0 * np.pi, perturb_modes)
        th = np.arctan2(x[:, 1], x[:, 0])
        s = np.zeros(x.shape[0])
        for k in range(perturb_modes):
            s += amp[k] * np.sin(m[k] * th + 2.0 * np.pi * nk[k] * x[:, 2] / length + phi[k])
        rwall_ratio = 1.0 + s
        x[:, 0] *= rwall_ratio
        x[:, 1] *= rwall_ratio
        params.update(amp=amp.tolist(), m=m.tolist(), n=nk.tolist(), phi=phi.tolist())

    # triangles of the cross-section: split each quad along alternating diagonals
    q = quads
    alt = (np.arange(q.shape[0]) % 2) == 0
    tA = np.where(alt[:, None], q[:, [0, 1, 2]], q[:, [0, 1, 3]])
    tB = np.where(alt[:, None], q[:, [0, 2, 3]], q[:, [1, 2, 3]])
    tri2d = np.concatenate([tA, tB], axis=0)
    ntri = tri2d.shape[0]
    nq_fluid = nc * nc + nr * 4 * nc
    tri_solid = (np.arange(ntri) % q.shape[0]) >= nq_fluid

    tets = []
    for k in range(nz):
        tets.append(_split_prisms(tri2d + k * nxy, tri2d + (k + 1) * nxy))
    ien = np.concatenate(tets, axis=0)
    ien = _orient(x, ien).astype(np.int32)
    nNo = x.shape[0]
    nEl = ien.shape[0]

    # faces
    per_layer = 3 * ntri
    elem_solid = np.tile(np.repeat(tri_solid, 3), nz)
    inlet_tri = tri2d[~tri_solid].copy()
    outlet_tri = tri2d[~tri_solid] + nz * nxy
    cand_in = np.arange(0, per_layer)
    cand_out = np.arange((nz - 1) * per_layer, nz * per_layer)
    gE_in = _match_faces(inlet_tri, ien, cand_in, nNo)
    gE_out = _match_faces(outlet_tri, ien, cand_out, nNo)

    wall_tri, gE_w = _loop_face(wall_loop, nz, nxy, ien, nNo, ~elem_solid)

    def face(name, tri, gE):
        return Face(name, tri.astype(np.int32), gE, np.unique(tri).astype(np.int32))

    faces = {"inlet": face("inlet", inlet_tri, gE_in), "outlet": face("outlet", outlet_tri, gE_out),
             "wall": face("wall", wall_tri, gE_w)}
    eid = None
    if nrs > 0:
        sin_tri = tri2d[tri_solid]
        sout_tri = tri2d[tri_solid] + nz * nxy
        faces["wall_inlet"] = face("wall_inlet", sin_tri, _match_faces(sin_tri, ien, cand_in, nNo))
        faces["wall_outlet"] = face("wall_outlet", sout_tri, _match_faces(sout_tri, ien, cand_out, nNo))
        otri, gE_o = _loop_face(outer_loop, nz, nxy, ien, nNo, elem_solid)
        faces["wall_outer"] = face("wall_outer", otri, gE_o)
        eid = np.where(elem_solid, 2, 1).astype(np.int32)
        params.update(nrs=nrs, thickness=thickness)
    gi = faces["inlet"].gN
    rr = np.hypot(x[gi, 0], x[gi, 1])
    rw = radius * rwall_ratio[gi]
    prof = np.clip(1.0 - (rr / rw) ** 2, 0.0, None)
    return PipeMesh(x=x, ien=ien, faces=faces, radius=radius, length=length,
                    inlet_profile=prof, params=params, eid=eid)


def _loop_face(L: np.ndarray, nz: int, nxy: int, ien: np.ndarray, nNo: int, elem_ok: np.ndarray):
    """Triangles of the cylindrical surface through the node loop ``L`` (quads between
    consecutive loop nodes of neighbouring layers, cut through their smallest node) and
    their owner tets among the elements flagged in ``elem_ok``."""
    nl = L.size
    wtris = []
    for k in range(nz):
        a = L + k * nxy
        b = np.roll(L, -1) + k * nxy
        a1 = a + nxy
        b1 = b + nxy
        Qd = np.stack([a, b, b1, a1], axis=1)
        mn = np.argmin(Qd, axis=1)
        # diagonal through the min node: min at 0 or 2 -> diag a-b1, else b-a1
        d02 = (mn == 0) | (mn == 2)
        t1 = np.where(d02[:, None], np.stack([a, b, b1], 1), np.stack([a, b, a1], 1))
        t2 = np.where(d02[:, None], np.stack([a, b1, a1], 1), np.stack([b, b1, a1], 1))
        wtris.append(t1)
        wtris.append(t2)
    tri = np.concatenate(wtris, axis=0)
    assert tri.shape[0] == 2 * nl * nz
    # candidate tets: those with at least 3 loop nodes
    on = np.zeros(nNo, dtype=bool)
    for k in range(nz + 1):
        on[L + k * nxy] = True
    cand = np.nonzero((on[ien].sum(axis=1) >= 3) & elem_ok)[0]
    return tri, _match_faces(tri, ien, cand, nNo)


# Named sizes.  'pipe50k' is the CPU-runnable case (~50k tets); 'pipe8m' the 8M-tet pipe
# with a seeded 8-mode wall perturbation; the others are test and sweep sizes.
SIZES = {
    "tiny": dict(nc=2, nr=1, nz=2),
    "small": dict(nc=4, nr=2, nz=6),
    "pipe50k": dict(nc=10, nr=6, nz=24),
    "pipe1m": dict(nc=20, nr=12, nz=120, perturb_modes=8),
    "pipe4m": dict(nc=32, nr=20, nz=180, perturb_modes=8),
    "pipe8m": dict(nc=40, nr=25, nz=240, perturb_modes=8),
    # FSI pipes: lumen plus a 1 mm solid wall annulus (radius 0.5 -> 0.6)
    "fsi_tiny": dict(nc=2, nr=1, nz=3, nrs=1),
    "fsi_small": dict(nc=4, nr=2, nz=6, nrs=2),
    # 4.0M fluid + 1.0M solid tets: the 4M + 1M-tet FSI pipe
    "fsi5m": dict(nc=32, nr=20, nz=186, nrs=7, perturb_modes=8),
}


def named_pipe(name: str) -> PipeMesh:
    return make_pipe(**SIZES[name])
