"""TEST INFRASTRUCTURE ONLY: numpy restatement of the reduced plume step
(SUBSPACE_FLUID_3D_EIGEN::stepReorderedCubatureStam).  Used by tests/ as the
checker of the GPU path (include/plume_reduced.h), never by the product.

The full-space part (velocity border wiped, buoyancy, vorticity confinement,
advectHeatAndDensityStam) is the C oracle's orc_reduced_prestep
(oracle/plume_oracle.cpp).  The reduced part follows
src/integrators/SUBSPACE_FLUID_3D_EIGEN.cpp:
  peeledProject        (VECTOR3_FIELD_3D.cpp:3434-3553)  q = U_pa^T peel(u)
  reducedAdvectStagedStamFast (1324-1350) with advectCellStamPeeled
                       (1106-1201): per cubature point the cell's velocity
                       from its cached 3 x r block, the backtrace clamped to
                       [1.5, res - 2.5], the trilinear weights, the eight
                       neighbours' U_pa rows times q, then the cached
                       weight x U_pd^T block; the points summed in order
  reducedPeeledDiffusion (606-612)   q = damping.peeled q
  reducedStagedProject   (700-707)   q = ptof q + inverseProduct q
  peeledUnproject      (VECTOR3_FIELD_3D.cpp:3558-3605)  interior u = U_f q
and readAdvectionCubature (1206-1319) for the cubature file; the cached
blocks are formed from U.preadvect and U.prediffuse as that function builds
them.
Parity of this restatement is pinned to the reference's own program
(oracle/_ref/reduced_ref) through tests/golden/ref_reduced_*.npz.
"""
import numpy as np


def read_matrix(path):
    """EIGEN::read: int32 rows, cols, then the row-major doubles."""
    raw = np.fromfile(path, dtype=np.uint8)
    rows, cols = np.frombuffer(raw[:8].tobytes(), dtype="<i4")
    return np.frombuffer(raw[8:].tobytes(), dtype="<f8").reshape(int(rows), int(cols))


def read_cubature(path):
    """The cubature file: int32 count, int32 peeled cells, double weights."""
    raw = open(path, "rb").read()
    n = int(np.frombuffer(raw[:4], dtype="<i4")[0])
    cells = np.frombuffer(raw[4:4 + 4 * n], dtype="<i4").astype(np.int64)
    weights = np.frombuffer(raw[4 + 4 * n:4 + 12 * n], dtype="<f8")
    return cells, weights


class ReducedModel:
    """The files the reference's constructor and loadReducedRuntimeBases read
    under a reduced path."""

    def __init__(self, path):
        d = path if path.endswith("/") else path + "/"
        self.Upa = read_matrix(d + "U.preadvect.matrix")
        self.Uf = read_matrix(d + "U.final.matrix")
        self.D = read_matrix(d + "damping.peeled.matrix")
        self.P = read_matrix(d + "projected.ptof.matrix")
        self.G = read_matrix(d + "inverseProduct.matrix")
        self.cells, weights = read_cubature(d + "cubature")
        # cellBasisPeeled blocks (lines 860-879): the cell's three rows
        rows = 3 * self.cells[:, None] + np.arange(3)[None, :]
        self.before = self.Upa[rows]                       # (points, 3, r_pa)
        Upd = read_matrix(d + "U.prediffuse.matrix")
        self.after = weights[:, None, None] * np.transpose(Upd[rows], (0, 2, 1))  # (points, r_pd, 3)


def _peel(res, u):
    X, Y, Z = res
    return u.reshape(Z, Y, X, 3)[1:-1, 1:-1, 1:-1].reshape(-1)


def step(o, model, res, dx):
    """One stepReorderedCubatureStam on the oracle handle `o`; returns q."""
    X, Y, Z = (int(v) for v in res)
    nx, ny = X - 2, Y - 2
    slab = nx * ny
    o.reduced_prestep()
    u = o.field("velocity")
    q = model.Upa.T @ _peel(res, u)
    dt0 = 0.1 / dx
    final = np.zeros(model.after.shape[1])
    for p, index in enumerate(model.cells):
        z = index // slab + 1
        y = (index % slab) // nx + 1
        x = (index % slab) % nx + 1
        v = model.before[p] @ q
        xt = min(max(x - dt0 * v[0], 1.5), X - 2.5)
        yt = min(max(y - dt0 * v[1], 1.5), Y - 2.5)
        zt = min(max(z - dt0 * v[2], 1.5), Z - 2.5)
        x0, y0, z0 = int(xt) - 1, int(yt) - 1, int(zt) - 1
        s1 = (xt - 1) - x0
        s0 = 1.0 - s1
        t1 = (yt - 1) - y0
        t0 = 1.0 - t1
        u1 = (zt - 1) - z0
        u0 = 1.0 - u1
        acc = np.zeros(3)
        for (dx_, dy_, dz_, w) in ((0, 0, 0, u0 * s0 * t0), (0, 1, 0, u0 * s0 * t1), (1, 0, 0, u0 * s1 * t0),
                                   (1, 1, 0, u0 * s1 * t1), (0, 0, 1, u1 * s0 * t0), (0, 1, 1, u1 * s0 * t1),
                                   (1, 0, 1, u1 * s1 * t0), (1, 1, 1, u1 * s1 * t1)):
            i = 3 * ((x0 + dx_) + (y0 + dy_) * nx + (z0 + dz_) * slab)
            acc += w * (model.Upa[i:i + 3] @ q)
        final += model.after[p] @ acc
    q = model.D @ final
    q = model.P @ q + model.G @ q
    # peeledUnproject: the interior from U_f q, the border as the prestep left it
    inner = (model.Uf @ q).reshape(Z - 2, Y - 2, X - 2, 3)
    full = u.reshape(Z, Y, X, 3).copy()
    full[1:-1, 1:-1, 1:-1] = inner
    o.set_field("velocity", full.reshape(-1))
    return q


def run(params, path, steps):
    """`steps` reduced steps from rest with the column source before each:
    (oracle handle, last q)."""
    from oracle import oracle
    o = oracle.Oracle(params)
    model = ReducedModel(path)
    res = tuple(int(v) for v in params.res)
    dx = 1.0 / max(res)
    q = None
    for s in range(steps):
        o.add_source(s)
        q = step(o, model, res, dx)
    return o, q

