"""Invariants of the reference's algorithm, checked on the oracle (CPU).

* ET-PL07 (edges_treatment.py:31-224): after the edge treatment the parabolas are continuous
  across each of the 12 cube edges (the two one-sided values are replaced by their mean on both
  sides) and every ghost cell holds its neighbour's boundary-cell parabola.  The reference keeps
  this check commented out (reconstruction_1d.py:397-483); here it runs for every reconstruction.
  The GPU staged engine matches the oracle's stage arrays (test_gpu_parity.py).
* Lagrange ghost-cell weights (lagrange.py:18-163): degree 3, so along the neighbour panel's
  edge-parallel coordinate they reproduce every cubic exactly (to rounding).
"""
import numpy as np
import pytest

from oracle import ppm
from oracle.grid import CubedSphere
from oracle.halo import CONNECT, E, N_, S, W, lagrange_tables


@pytest.mark.parametrize("recon", ["PPM-0", "PPM-CW84", "PPM-PL07", "PPM-L04"])
def test_pl07_parabolas_continuous_across_cube_edges(recon):
    g = CubedSphere(16)
    n = g.N + g.ng
    i0, iend, j0, jend = g.i0, g.iend, g.j0, g.jend
    Q = 1.0 + 0.3 * np.sin(2.0 * g.pc.lon) * np.cos(g.pc.lat) + 0.1 * g.pc.lat
    qLx, qRx, qLy, qRy = (np.zeros((n, n, 6)) for _ in range(4))
    ppm.reconstruct(Q, qLx, qRx, recon, i0, iend)
    ppm.reconstruct(ppm.T(Q), ppm.T(qLy), ppm.T(qRy), recon, j0, jend)
    ppm.edges_extrapolation(Q, Q, qLx, qRx, qLy, qRy, g, recon)
    cell, arrays = ppm._edge_refs(g, qLx, qRx, qLy, qRy)
    k = np.arange(i0, iend)
    facing = {E: W, W: E, N_: S, S: N_}
    for (p, s), (q, qs, rev) in CONNECT.items():
        kk = (n - 1 - k) if rev else k
        ep, _ = arrays(s)
        eq, fq = arrays(qs)
        # one value at the cube edge, seen from both panels
        np.testing.assert_array_equal(ep[cell(s, k, p)], eq[cell(qs, kk, q)])
        # the ghost cell beyond side s: the neighbour's parabola, its cube-edge value facing p
        gp_edge, gp_far = arrays(facing[s])
        np.testing.assert_array_equal(gp_edge[cell(s, k, p, ghost=True)], eq[cell(qs, kk, q)])
        np.testing.assert_array_equal(gp_far[cell(s, k, p, ghost=True)], fq[cell(qs, kk, q)])


@pytest.mark.parametrize("N", [16, 24, 41])
def test_lagrange_weights_reproduce_cubics(N):
    g = CubedSphere(N)
    Wt, Kmin = lagrange_tables(g)
    i0, iend, ngl = g.i0, g.iend, g.ngl
    pc = g.pc
    # the nodes: panel 1's angular coordinate of its cells at each depth; the targets: panel 0's
    # east ghost cells in that coordinate (the inverse map tan y = Z / Y, cs_transform.py:105-107)
    ys = np.arctan(pc.Z[i0:i0 + ngl, :, 1] / pc.Y[i0:i0 + ngl, :, 1])
    yg = np.arctan(pc.Z[iend:iend + ngl, :, 0] / pc.Y[iend:iend + ngl, :, 0])
    rng = np.random.default_rng(2)
    for _ in range(3):
        coef = rng.standard_normal(4)
        for d in range(ngl):
            for k in range(N + g.ng):
                nodes = ys[d, Kmin[d, k]:Kmin[d, k] + 4]
                got = np.dot(Wt[d, k], np.polynomial.polynomial.polyval(nodes, coef))
                want = np.polynomial.polynomial.polyval(yg[d, k], coef)
                assert abs(got - want) <= 1e-12 * (1.0 + abs(want)), (d, k)
