"""The problem of the reference's physics-based BDDC test (test 1 of
Sources/Tests/Scripts/par_test_pb_bddc_linear_elasticity:29): 20^3 trilinear hexahedra on
[0,2] x [0,0.5] x [0,0.5], Q1 linear elasticity, nu = 0.2, E = 1 outside and 1e8 inside the
channels of inclusion 7 (`-i 7 -nc 2 2 2 -npwc 2 2 2 -j 100000000`, 2 x 2 x 2 parts), zero
source, u = (x+y+z)(1,1,1) on the whole boundary.  CG with rtol 1e-6 printed the tolerance
3.708160389E+02 = 1e-6 ||b|| (Sources/Tests/Data/par_test_pb_bddc_linear_elasticity/
test1_convergence:1-13) and converged in 11 iterations.

Restated from the test driver (Sources/Tests/Par/par_test_pb_bddc_linear_elasticity/modules/
par_test_pb_bddc_linear_elasticity_driver.f90): channel positions :492-526, the x/y/z edge
channels :528-555 (a cell is in a channel when its vertex centroid lies in the closed box,
is_point_in_rectangle :722-737, set id 2 for every channel), boundary set ids :206-214; the
integrand (sbm_irreducible_heterogeneous_discrete_integration.i90:57-88: E = 1 for set ids
<= 1, else the jump; nu_heterogeneous = 0.2 in linear_elasticity_discrete_integration.f90:35),
the source (zero, linear_elasticity_analytical_functions.f90:99-112) and the boundary values
(the solution function, :128-142; linear_elasticity_conditions.f90: every boundary id
Dirichlet in every component).  Test infrastructure only.
"""
import numpy as np

N = (20, 20, 20)
LIMITS = (0.0, 2.0, 0.0, 0.5, 0.0, 0.5)
NCHANNEL = (2, 2, 2)
NPARTS_WITH_CHANNELS = (2, 2, 2)
NPARTS = (2, 2, 2)
JUMP = 1.0e8
NU = 0.2
RTOL = 1.0e-6
TOLERANCE = 3.708160389e02   # printed with 10 significant digits
ITERATIONS = 11
FIRST_RESIDUAL = 8.967533941e06  # the CG log's first error estimate (test1_convergence:2)


def _positions(d):
    lo, hi = LIMITS[2 * d], LIMITS[2 * d + 1]
    width = (hi - lo) * NPARTS_WITH_CHANNELS[d] / (NCHANNEL[d] * NPARTS[d])
    half = width / 5
    centre = half + lo
    p1, p2 = [], []
    for _ in range(NCHANNEL[d]):
        p1.append(centre - half)
        p2.append(centre + half)
        centre = centre + width
    return p1, p2


def _inside(origin, opposite, x):
    return all(not (x[i] < origin[i] or x[i] > opposite[i]) for i in range(3))


def cell_modulus():
    """E per cell, x fastest."""
    (px1, px2), (py1, py2), (pz1, pz2) = _positions(0), _positions(1), _positions(2)
    x0, x1, y0, y1, z0, z1 = LIMITS
    h = [(LIMITS[2 * d + 1] - LIMITS[2 * d]) / N[d] for d in range(3)]
    E = np.ones(N[0] * N[1] * N[2])
    for k in range(N[2]):
        for j in range(N[1]):
            for i in range(N[0]):
                verts = [(x0 + (i + a) * h[0], y0 + (j + b) * h[1], z0 + (k + c) * h[2])
                         for c in (0, 1) for b in (0, 1) for a in (0, 1)]
                x = [sum(v[d] for v in verts) / 8.0 for d in range(3)]
                inside = False
                for jj in range(NCHANNEL[1]):
                    for kk in range(NCHANNEL[2]):
                        inside |= _inside((x0, py1[jj], pz1[kk]), (x1, py2[jj], pz2[kk]), x)
                for jj in range(NCHANNEL[0]):
                    for kk in range(NCHANNEL[2]):
                        inside |= _inside((px1[jj], y0, pz1[kk]), (px2[jj], y1, pz2[kk]), x)
                for jj in range(NCHANNEL[0]):
                    for kk in range(NCHANNEL[1]):
                        inside |= _inside((px1[jj], py1[kk], z0), (px2[jj], py2[kk], z1), x)
                if inside:
                    E[i + N[0] * (j + N[1] * k)] = JUMP
    return E


def vertex_xyz():
    xs = [np.linspace(LIMITS[2 * d], LIMITS[2 * d + 1], N[d] + 1) for d in range(3)]
    Z, Y, X = np.meshgrid(xs[2], xs[1], xs[0], indexing="ij")
    return np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1).ravel()
