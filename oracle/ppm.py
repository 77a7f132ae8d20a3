"""PPM reconstruction, cube-edge treatment of parabolas, upwind fluxes (oracle restatement).

All 1-D operators act along axis 0 of an ``[i, j, p]`` array.  The y-direction versions
of the reference (``*_y``) are the same arithmetic on the transposed view
``A.transpose(1, 0, 2)``, which is how this module applies them.

* ``reconstruct``         -- reconstruction_1d.py:26-192 (PPM-0, PPM-PL07, PPM-CW84, PPM-L04)
* ``edges_extrapolation`` -- edges_treatment.py:82-178 (PL07 App. C, ET-PL07) incl.
                             ``average_parabola_cube_edges`` edges_treatment.py:31-76
* ``upwind_flux``         -- flux.py:20-70 (numerical_flux_ppm_x; _y by transposition)
* ``average_flux_cube_edges`` -- edges_treatment.py:231-278 (MF-AF)
"""
import numpy as np

from .halo import CONNECT, E, W, N_, S, flux_sign

RECON_NAMES = {1: "PPM-0", 2: "PPM-CW84", 3: "PPM-PL07", 4: "PPM-L04"}


def T(a):
    """y-direction view: swap the first two axes."""
    return a.transpose(1, 0, 2)


def reconstruct(Q, qL, qR, name, i0, iend):
    """Edge values qL, qR of cells [i0-1, iend] along axis 0 (reconstruction_1d.py:26-192)."""
    n0 = Q.shape[0]
    c = slice(i0 - 1, iend + 1)
    if name == "PPM-0":
        Qe = np.zeros((n0 + 1,) + Q.shape[1:])
        e = np.arange(i0 - 1, iend + 2)
        Qe[e] = (7.0 / 12.0) * (Q[e] + Q[e - 1]) - (Q[e + 1] + Q[e - 2]) / 12.0
        qR[c] = Qe[i0:iend + 2]
        qL[c] = Qe[i0 - 1:iend + 1]
    elif name == "PPM-PL07":
        a1, a2, a3, a4, a5 = 2.0 / 60.0, -13.0 / 60.0, 47.0 / 60.0, 27.0 / 60.0, -3.0 / 60.0
        q1, q2, q3 = Q[i0 - 3:iend - 1], Q[i0 - 2:iend], Q[i0 - 1:iend + 1]
        q4, q5 = Q[i0:iend + 2], Q[i0 + 1:iend + 3]
        qR[c] = a1 * q1 + a2 * q2 + a3 * q3 + a4 * q4 + a5 * q5
        qL[c] = a5 * q1 + a4 * q2 + a3 * q3 + a2 * q4 + a1 * q5
    elif name == "PPM-CW84":
        k = np.arange(i0 - 2, iend + 2)
        dQ = np.zeros_like(Q)
        d0 = 0.5 * (Q[k + 1] - Q[k - 1])
        d1 = 2.0 * (Q[k + 1] - Q[k])
        d2 = 2.0 * (Q[k] - Q[k - 1])
        s = np.minimum(np.abs(d0), np.abs(d1))
        s = np.minimum(s, np.abs(d2)) * np.sign(d0)
        mono = (Q[k + 1] - Q[k]) * (Q[k] - Q[k - 1]) > 0.0
        s[~mono] = 0.0
        dQ[k] = s
        Qe = np.zeros((n0 + 1,) + Q.shape[1:])
        e = np.arange(i0 - 1, iend + 2)
        Qe[e] = 0.5 * (Q[e] + Q[e - 1]) - (dQ[e] - dQ[e - 1]) / 6.0
        qR[c] = Qe[i0:iend + 2]
        qL[c] = Qe[i0 - 1:iend + 1]
        q = Q[c]
        R, L = qR[c], qL[c]  # views
        dq = R - L
        q6 = 6 * q - 3 * (R + L)
        lmax = (R - q) * (q - L) <= 0
        R[lmax] = q[lmax]
        L[lmax] = q[lmax]
        over = np.abs(dq) < np.abs(q6)
        mleft = (R - L) * (q - 0.5 * (R + L)) > ((R - L) ** 2) / 6.0
        mright = -((R - L) ** 2) / 6.0 > (R - L) * (q - 0.5 * (R + L))
        ml = over & mleft
        mr = over & mright
        L[ml] = 3.0 * q[ml] - 2.0 * R[ml]
        R[mr] = 3.0 * q[mr] - 2.0 * L[mr]
    elif name == "PPM-L04":
        k = np.arange(i0 - 3, iend + 3)
        dq = 0.25 * (Q[k + 1] - Q[k - 1])
        qmax = np.maximum(np.maximum(Q[k - 1], Q[k]), Q[k + 1])
        qmin = np.minimum(np.minimum(Q[k - 1], Q[k]), Q[k + 1])
        dmin = qmax - Q[k]
        dmax = Q[k] - qmin
        mono = np.zeros_like(Q)
        mono[k] = np.minimum(np.minimum(np.abs(dq), dmin), dmax) * np.sign(dq)
        Qe = np.zeros((n0 + 1,) + Q.shape[1:])
        e = np.arange(i0 - 1, iend + 2)
        Qe[e] = 0.5 * (Q[e] + Q[e - 1]) - (mono[e] - mono[e - 1]) / 3.0
        qR[c] = Qe[i0:iend + 2]
        qL[c] = Qe[i0 - 1:iend + 1]
        q0 = Q[c]
        m = mono[c]
        lim = np.minimum(2.0 * np.abs(m), np.abs(qL[c] - q0)) * np.sign(2.0 * m)
        qL[c] = q0 - lim
        lim = np.minimum(2.0 * np.abs(m), np.abs(qR[c] - q0)) * np.sign(2.0 * m)
        qR[c] = q0 + lim
    else:
        raise ValueError(name)


def _edge_refs(grid, qLx, qRx, qLy, qRy):
    """Accessors for the boundary-cell parabola of each panel side.

    Returns, for a side, (array, index builder, edge-side array, far-side array) such that
    the value at the cube edge and at the opposite face of the boundary cell can be read
    or written for an along-edge index vector.
    """
    i0, iend, j0, jend = grid.i0, grid.iend, grid.j0, grid.jend

    def cell(side, k, p, ghost=False):
        if side == E:
            return (iend if ghost else iend - 1, k, p)
        if side == W:
            return (i0 - 1 if ghost else i0, k, p)
        if side == N_:
            return (k, jend if ghost else jend - 1, p)
        return (k, j0 - 1 if ghost else j0, p)

    def arrays(side):
        # (edge-side array, far-side array) for the boundary cell of ``side``
        if side == E:
            return qRx, qLx
        if side == W:
            return qLx, qRx
        if side == N_:
            return qRy, qLy
        return qLy, qRy

    return cell, arrays


def edges_extrapolation(Qx, Qy, qLx, qRx, qLy, qRy, grid, recon_name):
    """ET-PL07 edge treatment of the parabolas (edges_treatment.py:82-178, 31-76)."""
    i0, iend, j0, jend = grid.i0, grid.iend, grid.j0, grid.jend
    n = grid.N + grid.ng
    for Qa, L, R in ((Qx, qLx, qRx), (T(Qy), T(qLy), T(qRy))):
        J = slice(j0, jend)
        L[i0, J] = 1.5 * Qa[i0, J] - 0.5 * Qa[i0 + 1, J]
        R[iend - 1, J] = 1.5 * Qa[iend - 1, J] - 0.5 * Qa[iend - 2, J]
        R[i0, J] = (3.0 * Qa[i0, J] + 11.0 * Qa[i0 + 1, J] - 2.0 * (Qa[i0 + 2, J] - Qa[i0, J])) / 14.0
        L[i0 + 1, J] = R[i0, J]
        L[iend - 1, J] = (3.0 * Qa[iend - 1, J] + 11.0 * Qa[iend - 2, J]
                          - 2.0 * (Qa[iend - 3, J] - Qa[iend - 1, J])) / 14.0
        R[iend - 2, J] = L[iend - 1, J]
        if recon_name == "PPM-PL07":
            R[i0 + 1, J] = L[i0 + 2, J]
            L[iend - 2, J] = R[iend - 3, J]
    cell, arrays = _edge_refs(grid, qLx, qRx, qLy, qRy)
    k = np.arange(i0, iend)
    done = set()
    # average the two one-sided values at each of the 12 cube edges
    for (p, s), (q, qs, rev) in CONNECT.items():
        if (q, qs) in done:
            continue
        done.add((p, s))
        kk = (n - 1 - k) if rev else k
        ep, _ = arrays(s)
        eq, _ = arrays(qs)
        v = (ep[cell(s, k, p)] + eq[cell(qs, kk, q)]) * 0.5
        ep[cell(s, k, p)] = v
        eq[cell(qs, kk, q)] = v
    # copy the neighbour's boundary-cell parabola into each ghost cell
    upd = []
    for (p, s), (q, qs, rev) in CONNECT.items():
        kk = (n - 1 - k) if rev else k
        eq, fq = arrays(qs)
        upd.append((p, s, eq[cell(qs, kk, q)].copy(), fq[cell(qs, kk, q)].copy()))
    for p, s, ev, fv in upd:
        # for the ghost cell of side s, the cube edge is on the side facing the panel
        ep, fp = arrays(W if s == E else E if s == W else S if s == N_ else N_)
        ep[cell(s, k, p, ghost=True)] = ev
        fp[cell(s, k, p, ghost=True)] = fv


def upwind_flux(Qa, L, R, cx, uavg, upos, g_pu, g_pc, mt_name, i0, iend):
    """PPM upwind flux at edges [i0, iend] along axis 0 (flux.py:20-70).

    ``L``/``R`` are modified in place by the MT-0 metric factor, as in the reference.
    Returns f_upw for edges [i0, iend] (shape (N+1, ...)).
    """
    c = slice(i0 - 1, iend + 1)
    if mt_name == "MT-0":
        L[c] = L[c] * g_pu[i0 - 1:iend + 1]
        R[c] = R[c] * g_pu[i0:iend + 2]
        q = Qa[c] * g_pc[c]
    else:
        q = Qa[c]
    dq = R[c] - L[c]
    q6 = 6 * q - 3 * (R[c] + L[c])
    # dq, q6 indexed by cell - (i0 - 1)
    e = slice(i0, iend + 1)
    cc = cx[e]
    fl = R[i0 - 1:iend] + cc * 0.5 * (q6[0:-1] - dq[0:-1]) - q6[0:-1] * cc * cc / 3.0
    fr = L[i0:iend + 1] - cc * 0.5 * (q6[1:] + dq[1:]) - q6[1:] * cc * cc / 3.0
    f = np.where(upos, fl, fr)
    f = f * uavg[e]
    if mt_name == "MT-PL07":
        f = f * g_pu[e]
    return f


def average_flux_cube_edges(fx, fy, grid):
    """MF-AF: average the two panels' upwind fluxes at each cube edge (edges_treatment.py:231-278)."""
    i0, iend, j0, jend = grid.i0, grid.iend, grid.j0, grid.jend
    n = grid.N + grid.ng
    k = np.arange(i0, iend)

    def ref(side, kk, p):
        if side == E:
            return fx, (iend, kk, p)
        if side == W:
            return fx, (i0, kk, p)
        if side == N_:
            return fy, (kk, jend, p)
        return fy, (kk, j0, p)

    done = set()
    for (p, s), (q, qs, rev) in CONNECT.items():
        if (q, qs) in done:
            continue
        done.add((p, s))
        kk = (n - 1 - k) if rev else k
        sg = flux_sign(s, qs)
        ap, ip = ref(s, k, p)
        aq, iq = ref(qs, kk, q)
        if sg > 0:
            v = 0.5 * ap[ip] + 0.5 * aq[iq]
            ap[ip] = v
            aq[iq] = v
        else:
            v = 0.5 * ap[ip] - 0.5 * aq[iq]
            ap[ip] = v
            aq[iq] = -v
