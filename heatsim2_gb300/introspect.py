"""Reference-form stage matrices rebuilt from a compiled problem, for inspection and tests.

``stage_matrices(params, s)`` returns what the reference's ``pyadi_step`` holds after ``finalize``
(alternatingdirection_c_pyx.pyx:212-282): the tridiagonal ``A`` (n x 3, rows in stage s's permuted order),
sparse ``B`` and ``C_j`` (scipy CSR, rows and columns permuted), ``D``, and the ``tridiaglu`` factors
``L``/``U`` (tridiag.pyx:9-43).  The GPU step does not use these: it solves the same stage equations in the
scaled delta form compiled on the device.
"""
import numpy as np

_STAGE_OF_AXIS = (2, 1, 0)      # z is solved last, x first (alternatingdirection_c_pyx.pyx:426-432)
_PERMS = ((0, 1, 2), (2, 0, 1), (1, 2, 0))


def _own_face_conductances(params):
    """Per-voxel G_lo, G_hi for each axis seen from the voxel's own equation (zero for fixed voxels)."""
    Gz, Gy, Gx, M, fixed = params.faces()
    comp = fixed == 0
    lo = [Gz[:-1], Gy[:, :-1], Gx[:, :, :-1]]
    hi = [Gz[1:], Gy[:, 1:], Gx[:, :, 1:]]
    lo = [np.where(comp, g, 0.0) for g in lo]
    hi = [np.where(comp, g, 0.0) for g in hi]
    return lo, hi, M, comp


def _tridiaglu(A):
    n = A.shape[0]
    L = np.zeros((n, 3))
    U = A.copy()
    for row in range(n):
        L[row, 1] = U[row, 1]
        U[row, 2] /= U[row, 1]
        U[row, 1] = 1.0
        if row < n - 1:
            coef = U[row + 1, 0]
            U[row + 1, 0] = 0.0
            U[row + 1, 1] -= U[row, 2] * coef
            L[row + 1, 0] = coef
    return L, U


def stage_matrices(params, s, factor=True):
    import scipy.sparse
    nz, ny, nx = params.shape
    n = nz * ny * nx
    lo, hi, M, comp = _own_face_conductances(params)
    perm = _PERMS[s]
    # permuted row number of every voxel (natural order in, permuted index out)
    pidx = np.arange(n).reshape(nz, ny, nx).transpose(perm).reshape(n)
    rowof = np.empty(n, dtype=np.int64)
    rowof[pidx] = np.arange(n)
    rowof = rowof.reshape(nz, ny, nx)
    rows, cols, vals = [], [], []
    crow = [[] for _ in range(s)]
    ccol = [[] for _ in range(s)]
    cval = [[] for _ in range(s)]
    A = np.zeros((n, 3))
    center = np.where(comp, M, 1.0).astype("d")
    diag = center.copy()
    sa = 2 - s                       # axis solved in this stage
    shifts = ((1, 0, 0), (0, 1, 0), (0, 0, 1))
    r_all = rowof
    for a in range(3):
        st = _STAGE_OF_AXIS[a]
        w = 0.5 if st <= s else 1.0
        for side, G in ((-1, lo[a]), (1, hi[a])):
            mask = G != 0.0
            if not mask.any():
                continue
            k, j, i = np.nonzero(mask)
            q = [k, j, i]
            q[a] = q[a] + side
            g = G[mask]
            r = r_all[k, j, i]
            c = r_all[q[0], q[1], q[2]]
            rows.append(r)
            cols.append(c)
            vals.append(w * g)
            center[k, j, i] -= w * g
            if a == sa:
                A[r, 1 + side] = -(0.5 * g)
                diag[k, j, i] += 0.5 * g
            elif st < s:
                crow[st] += [r, r]
                ccol[st] += [c, r]
                cval[st] += [0.5 * g, -(0.5 * g)]
    rows.append(r_all.reshape(n))
    cols.append(r_all.reshape(n))
    vals.append(center.reshape(n))
    A[r_all.reshape(n), 1] = diag.reshape(n)
    B = scipy.sparse.coo_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                                shape=(n, n)).tocsr()
    C = []
    for st in range(s):
        if crow[st]:
            C.append(scipy.sparse.coo_matrix((np.concatenate([np.atleast_1d(v) for v in cval[st]]),
                                              (np.concatenate([np.atleast_1d(v) for v in crow[st]]),
                                               np.concatenate([np.atleast_1d(v) for v in ccol[st]]))),
                                             shape=(n, n)).tocsr())
        else:
            C.append(scipy.sparse.csr_matrix((n, n)))
    D = np.zeros(n)
    D[r_all.reshape(n)] = comp.reshape(n).astype("d")
    out = {"A": A, "B": B, "C": C, "D": D}
    if factor:
        out["L"], out["U"] = _tridiaglu(A)
    return out
