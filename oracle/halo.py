"""Ghost cells across cube edges (oracle restatement).

The reference hard-codes, per panel, numpy slices + transposes + flips that gather four
rows of a neighbouring panel (halo_data.py:15-400).  Here the same connectivity is a
table: for panel ``p`` and side ``s`` it gives the neighbour ``q``, the side of ``q``
that touches ``p`` and whether the along-edge index runs backwards.  A ghost cell at
depth ``d`` (0 = next to the edge) outside side ``s`` of ``p`` maps to the cell at depth
``d`` inside side ``qs`` of ``q``.  The table was derived from halo_data.py:33-182 and is
checked against the reference's gathers in the golden tests.

Functions:
* ``lagrange_tables``          -- degree-3 ghost-cell weights and stencils, lagrange.py:18-163
* ``dg_fill``                  -- ET-DG scalar fill, interpolation.py:154-314
* ``adjacent_fill``            -- ET-S72/ET-PL07 copy, interpolation.py:320-340
* ``vector_halo_dg``           -- ET-DG wind halo, interpolation.py:347-532
* ``vector_halo_adjacent_rk2`` -- ET-S72/ET-PL07 + RK2 wind copy, edges_treatment.py:305-347
"""
import math

import numpy as np

E, W, N_, S = 0, 1, 2, 3
SIDE_NAMES = ("E", "W", "N", "S")

# (p, side) -> (q, side of q, reversed along-edge index)
CONNECT = {
    (0, E): (1, W, 0), (0, W): (3, E, 0), (0, N_): (4, S, 0), (0, S): (5, N_, 0),
    (1, E): (2, W, 0), (1, W): (0, E, 0), (1, N_): (4, E, 0), (1, S): (5, E, 1),
    (2, E): (3, W, 0), (2, W): (1, E, 0), (2, N_): (4, N_, 1), (2, S): (5, S, 1),
    (3, E): (0, W, 0), (3, W): (2, E, 0), (3, N_): (4, W, 1), (3, S): (5, W, 0),
    (4, E): (1, N_, 0), (4, W): (3, N_, 1), (4, N_): (2, N_, 1), (4, S): (0, N_, 0),
    (5, E): (1, S, 1), (5, W): (3, S, 0), (5, N_): (0, S, 0), (5, S): (2, S, 1),
}


def side_sign(side):
    """+1 if the outward normal of ``side`` is the positive coordinate direction."""
    return 1 if side in (E, N_) else -1


def flux_sign(p_side, q_side):
    """Sign relating p's coordinate direction to q's across a shared edge.

    Used for vector quantities (edge winds, fluxes): edges_treatment.py:241-278, 311-347.
    """
    return -side_sign(p_side) * side_sign(q_side)


def inside_index(grid, side, d, k):
    """(i, j) of the cell at depth d inside ``side``, along-edge index k (arrays ok)."""
    i0, iend, j0, jend = grid.i0, grid.iend, grid.j0, grid.jend
    if side == W:
        return i0 + d, k
    if side == E:
        return iend - 1 - d, k
    if side == S:
        return k, j0 + d
    return k, jend - 1 - d


def ghost_index(grid, side, d, k):
    """(i, j) of the ghost cell at depth d outside ``side``, along-edge index k."""
    i0, iend, j0, jend = grid.i0, grid.iend, grid.j0, grid.jend
    if side == E:
        return iend + d, k
    if side == W:
        return i0 - 1 - d, k
    if side == N_:
        return k, jend + d
    return k, j0 - 1 - d


def lagrange_tables(grid, degree=3):
    """Ghost-cell Lagrange weights and stencil starts (lagrange.py:18-163).

    Built once for panel 0's east ghost cells expressed in panel 1's angular coordinate
    and reused (by symmetry) for every panel and side.  Returns ``(W, Kmin)`` with shapes
    (4, N+8, degree+1) and (4, N+8), indexed by [depth, along-edge index].
    """
    N, ng, ngl = grid.N, grid.ng, grid.ngl
    i0, iend = grid.i0, grid.iend
    dy = grid.dy
    order = degree + 1
    pc = grid.pc
    # inverse equiangular map for panel 1: tan y = Z / Y (cs_transform.py:105-107)
    yg = np.arctan(pc.Z[iend:iend + ngl, :, 0] / pc.Y[iend:iend + ngl, :, 0])
    ys = np.arctan(pc.Z[i0:i0 + ngl, :, 1] / pc.Y[i0:i0 + ngl, :, 1])
    Kmin = np.zeros((ngl, N + ng), dtype=np.int64)
    for g in range(ngl):
        for k in range(N + ng):
            K = (yg[g, k] - ys[g, 0]) / dy
            kmax = K + math.ceil(order / 2)
            kmin = kmax - order + 1
            if i0 <= k < iend:
                if kmax >= iend:
                    kmax = iend - 1
                    kmin = kmax - order + 1
                elif kmin < i0:
                    kmin = i0
                    kmax = kmin + order - 1
            elif k >= iend:
                if kmax >= N + ng:
                    kmax = N + ng - 1
                    kmin = kmax - order + 1
            else:
                if kmin < 0:
                    kmin = 0
                    kmax = kmin + order - 1
            Kmin[g, k] = int(kmin)
            if int(kmax) - int(kmin) != degree:
                raise RuntimeError("inconsistent Lagrange stencil")
    Wt = np.zeros((ngl, N + ng, order))
    for g in range(ngl):
        for k in range(N + ng):
            nodes = ys[g, Kmin[g, k]:Kmin[g, k] + order]
            x = yg[g, k]
            for l in range(order):
                L = 1.0
                for m in range(order):
                    if m != l:
                        L = L * (x - nodes[m]) / (nodes[l] - nodes[m])
                Wt[g, k, l] = L
    # stencil checks of lagrange.py:110-126 (interior along-edge positions)
    for g in range(ngl):
        for k in range(i0, iend):
            if Kmin[g, k] < i0 or Kmin[g, k] + degree > iend:
                raise RuntimeError("Lagrange stencil leaves the panel")
    return Wt, Kmin


def gather(F, grid, p, side):
    """Neighbour data for ghost cells of (p, side): H[d, k], d<4, k<N+8 (halo_data.py:15-185)."""
    q, qs, rev = CONNECT[(p, side)]
    n = grid.N + grid.ng
    k = np.arange(n)
    kk = (n - 1 - k) if rev else k
    H = np.empty((grid.ngl, n))
    for d in range(grid.ngl):
        ii, jj = inside_index(grid, qs, d, kk)
        H[d] = F[ii, jj, q]
    return H


def _lagrange_apply(H, Wt, Kmin, ks):
    """sum_m W[d,k,m] * H[d, Kmin[d,k]+m], products then a left-to-right sum."""
    nd = H.shape[0]
    out = np.empty((nd, len(ks)))
    for d in range(nd):
        idx = Kmin[d, ks][:, None] + np.arange(Wt.shape[2])[None, :]
        prod = H[d][idx] * Wt[d, ks, :]
        acc = prod[:, 0] + prod[:, 1]
        for m in range(2, Wt.shape[2]):
            acc = acc + prod[:, m]
        out[d] = acc
    return out


def dg_fill(F, grid, Wt, Kmin):
    """ET-DG: fill every ghost cell of F by Lagrange interpolation (interpolation.py:154-314).

    First the four side strips of every panel from the neighbours' interior rows, then the
    four 4x4 corner blocks from the refreshed halo of the east and west neighbours.
    """
    j0, jend = grid.j0, grid.jend
    n = grid.N + grid.ng
    interior = np.arange(j0, jend)
    H = {(p, s): gather(F, grid, p, s) for p in range(6) for s in range(4)}
    for p in range(6):
        for s in range(4):
            vals = _lagrange_apply(H[(p, s)], Wt, Kmin, interior)
            for d in range(grid.ngl):
                ii, jj = ghost_index(grid, s, d, interior)
                F[ii, jj, p] = vals[d]
    corners = np.concatenate([np.arange(0, j0), np.arange(jend, n)])
    H = {(p, s): gather(F, grid, p, s) for p in range(6) for s in (E, W)}
    for p in range(6):
        for s in (E, W):
            vals = _lagrange_apply(H[(p, s)], Wt, Kmin, corners)
            for d in range(grid.ngl):
                ii, jj = ghost_index(grid, s, d, corners)
                F[ii, jj, p] = vals[d]


def adjacent_fill(Qx, Qy, grid):
    """ET-S72/ET-PL07: copy neighbour cells into ghost cells (interpolation.py:320-340).

    East/west ghosts go to Qy, north/south ghosts to Qx; the source is the neighbour's Qy
    when the shared side is its east/west side, its Qx otherwise (halo_data.py:191-400).
    All data is gathered before any ghost cell is written; then Qy's west/east and Qx's
    south/north strips are written in that order (Qx may be Qy).
    """
    n = grid.N + grid.ng
    k = np.arange(n)
    data = {}
    for p in range(6):
        for s in (W, E, S, N_):
            q, qs, rev = CONNECT[(p, s)]
            src = Qy if qs in (E, W) else Qx
            data[(p, s)] = gather(src, grid, p, s)
    for dst, sides in ((Qy, (W, E)), (Qx, (S, N_))):
        for s in sides:
            for p in range(6):
                for d in range(grid.ngl):
                    ii, jj = ghost_index(grid, s, d, k)
                    dst[ii, jj, p] = data[(p, s)][d]


def vector_halo_adjacent_rk2(ucontra_pu, vcontra_pv, grid):
    """ET-S72/ET-PL07 + RK2: copy contravariant edge winds across cube edges.

    The edge one beyond each cube edge takes the neighbour's edge one inside, with the
    sign flip of rotated panel pairs (edges_treatment.py:305-347).
    """
    i0, iend, j0, jend = grid.i0, grid.iend, grid.j0, grid.jend
    n = grid.N + grid.ng
    k = np.arange(i0, iend)

    def edge_one_inside(q, qs, kk):
        if qs == W:
            return ucontra_pu[i0 + 1, kk, q]
        if qs == E:
            return ucontra_pu[iend - 1, kk, q]
        if qs == S:
            return vcontra_pv[kk, j0 + 1, q]
        return vcontra_pv[kk, jend - 1, q]

    vals = {}
    for p in range(6):
        for s in range(4):
            q, qs, rev = CONNECT[(p, s)]
            kk = (n - 1 - k) if rev else k
            vals[(p, s)] = flux_sign(s, qs) * edge_one_inside(q, qs, kk)
    for (p, s), v in vals.items():
        if s == E:
            ucontra_pu[iend + 1, k, p] = v
        elif s == W:
            ucontra_pu[i0 - 1, k, p] = v
        elif s == N_:
            vcontra_pv[k, jend + 1, p] = v
        else:
            vcontra_pv[k, j0 - 1, p] = v


def latlon_to_contravariant(u, v, ps, idx):
    """sphgeo.py:120-125 at grid points ps[idx]."""
    uc = ps.ey_elat[idx] * u - ps.ey_elon[idx] * v
    vc = -ps.ex_elat[idx] * u + ps.ex_elon[idx] * v
    return uc / ps.det[idx], vc / ps.det[idx]


def contravariant_to_latlon(uc, vc, ps, idx):
    """sphgeo.py:130-133 at grid points ps[idx]."""
    return ps.ex_elon[idx] * uc + ps.ey_elon[idx] * vc, ps.ex_elat[idx] * uc + ps.ey_elat[idx] * vc


def vector_halo_dg(w, grid, Wt, Kmin):
    """ET-DG wind halo (interpolation.py:347-532).

    ``w`` holds the wind arrays: ``u_pu``/``v_pv`` (contravariant winds at x/y edges),
    ``ulon_pu``/``vlat_pu``/``ulon_pv``/``vlat_pv`` (lat-lon winds at edges) and
    ``uc_pc``/``vc_pc``/``ulon_pc``/``vlat_pc`` (at centres).  Steps:
    1. cubic edge->centre interpolation of the contravariant wind in a band of 4 cells
       along every panel boundary;
    2. contravariant->lat-lon at interior centres;
    3. Lagrange ghost fill of the lat-lon centre winds (dg_fill);
    4. cubic centre->edge interpolation at ghost edges and lat-lon->contravariant.
    """
    i0, iend, j0, jend = grid.i0, grid.iend, grid.j0, grid.jend
    ngl = grid.ngl
    U = w["u_pu"]
    V = w["v_pv"]
    uc, vc = w["uc_pc"], w["vc_pc"]
    a1, a2, a3, a4 = 5.0 / 16.0, 15.0 / 16.0, -5.0 / 16.0, 1.0 / 16.0
    b1, b2, b3, b4 = -1.0 / 16.0, 9.0 / 16.0, 9.0 / 16.0, -1.0 / 16.0
    J = slice(j0, jend)
    I = slice(i0, iend)
    # west band
    uc[i0, J] = a1 * U[i0, J] + a2 * U[i0 + 1, J] + a3 * U[i0 + 2, J] + a4 * U[i0 + 3, J]
    c = np.arange(i0 + 1, i0 + ngl)
    uc[c, J] = (b1 * U[c - 1, J] + b2 * U[c, J] + b3 * U[c + 1, J] + b4 * U[c + 2, J])
    cj = np.arange(j0 + ngl, jend - ngl)
    rows = slice(i0, i0 + ngl)
    vc[rows, cj] = (b1 * V[rows, cj - 1] + b2 * V[rows, cj] + b3 * V[rows, cj + 1] + b4 * V[rows, cj + 2])
    # east band
    uc[iend - 1, J] = a4 * U[iend - 3, J] + a3 * U[iend - 2, J] + a2 * U[iend - 1, J] + a1 * U[iend, J]
    c = np.arange(iend - ngl, iend - 1)
    uc[c, J] = (b4 * U[c - 1, J] + b3 * U[c, J] + b2 * U[c + 1, J] + b1 * U[c + 2, J])
    rows = slice(iend - ngl, iend)
    vc[rows, cj] = (b1 * V[rows, cj - 1] + b2 * V[rows, cj] + b3 * V[rows, cj + 1] + b4 * V[rows, cj + 2])
    # south band
    vc[I, j0] = a1 * V[I, j0] + a2 * V[I, j0 + 1] + a3 * V[I, j0 + 2] + a4 * V[I, j0 + 3]
    c = np.arange(j0 + 1, j0 + ngl)
    vc[I, c] = (b1 * V[I, c - 1] + b2 * V[I, c] + b3 * V[I, c + 1] + b4 * V[I, c + 2])
    ci = np.arange(i0 + ngl, iend - ngl)
    cols = slice(j0, j0 + ngl)
    uc[ci, cols] = (b1 * U[ci - 1, cols] + b2 * U[ci, cols] + b3 * U[ci + 1, cols] + b4 * U[ci + 2, cols])
    # north band
    vc[I, jend - 1] = a4 * V[I, jend - 3] + a3 * V[I, jend - 2] + a2 * V[I, jend - 1] + a1 * V[I, jend]
    c = np.arange(jend - ngl, jend - 1)
    vc[I, c] = (b4 * V[I, c - 1] + b3 * V[I, c] + b2 * V[I, c + 1] + b1 * V[I, c + 2])
    cols = slice(jend - ngl, jend)
    uc[ci, cols] = (b1 * U[ci - 1, cols] + b2 * U[ci, cols] + b3 * U[ci + 1, cols] + b4 * U[ci + 2, cols])
    # contravariant -> lat-lon at interior centres
    idx = (I, J, slice(None))
    w["ulon_pc"][idx], w["vlat_pc"][idx] = contravariant_to_latlon(uc[idx], vc[idx], grid.pc, idx)
    dg_fill(w["ulon_pc"], grid, Wt, Kmin)
    dg_fill(w["vlat_pc"], grid, Wt, Kmin)
    ul, vl = w["ulon_pc"], w["vlat_pc"]
    c1, c2 = 9.0 / 16.0, -1.0 / 16.0

    def to_contra_pu(idx):
        U[idx], w["vc_pu"][idx] = latlon_to_contravariant(w["ulon_pu"][idx], w["vlat_pu"][idx], grid.pu, idx)

    def to_contra_pv(idx):
        w["uc_pv"][idx], V[idx] = latlon_to_contravariant(w["ulon_pv"][idx], w["vlat_pv"][idx], grid.pv, idx)

    e = np.arange(i0, iend + 1)
    for cols in (slice(0, j0), slice(jend, None)):
        for src, dst in ((ul, "ulon_pu"), (vl, "vlat_pu")):
            w[dst][e, cols] = c1 * (src[e, cols] + src[e - 1, cols]) + c2 * (src[e + 1, cols] + src[e - 2, cols])
        to_contra_pu((e[:, None], np.arange(grid.N + grid.ng)[cols][None, :], slice(None)))
    e = np.arange(j0, jend + 1)
    for rows in (slice(0, i0), slice(iend, None)):
        for src, dst in ((ul, "ulon_pv"), (vl, "vlat_pv")):
            w[dst][rows, e] = c1 * (src[rows, e] + src[rows, e - 1]) + c2 * (src[rows, e + 1] + src[rows, e - 2])
        to_contra_pv((np.arange(grid.N + grid.ng)[rows][:, None], e[None, :], slice(None)))
    # edges one beyond the cube edges (used by the RK2 departure point)
    for dst, src in (("ulon_pu", ul), ("vlat_pu", vl)):
        w[dst][i0 - 1] = c1 * (src[i0 - 2] + src[i0 - 1]) + c2 * (src[i0] + src[i0 - 3])
    to_contra_pu((i0 - 1, slice(None), slice(None)))
    for dst, src in (("ulon_pu", ul), ("vlat_pu", vl)):
        w[dst][iend + 1] = c1 * (src[iend] + src[iend + 1]) + c2 * (src[iend - 1] + src[iend + 2])
    to_contra_pu((iend + 1, slice(None), slice(None)))
    for dst, src in (("ulon_pv", ul), ("vlat_pv", vl)):
        w[dst][:, j0 - 1] = c1 * (src[:, j0 - 2] + src[:, j0 - 1]) + c2 * (src[:, j0] + src[:, j0 - 3])
    to_contra_pv((slice(None), j0 - 1, slice(None)))
    for dst, src in (("ulon_pv", ul), ("vlat_pv", vl)):
        w[dst][:, jend + 1] = c1 * (src[:, jend] + src[:, jend + 1]) + c2 * (src[:, jend - 1] + src[:, jend + 2])
    to_contra_pv((slice(None), jend + 1, slice(None)))
