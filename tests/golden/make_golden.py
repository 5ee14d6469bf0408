"""Generate the committed fixtures under tests/golden/.

1. Decode the reference's own PETSc-binary test inputs (read from the reference
   checkout given as the first command-line argument, which is required) into .npz files:
   * utopia/data/laplace/matrices_for_petsc/{f_A, f_rhs, I_1, I_2, I_3}: the 4-level
     2D hierarchy of petsc_cg_mg / petsc_mg_jacobi
     (utopia/tests/petsc/utopia_PetscLinearSolverTest.cpp:400-508)
   * utopia/data/mg/{A.bin, I.bin, rhs.bin}: the 2-level case of petsc_mg
2. Record oracle regression pins (iteration counts, Galerkin structure digests) for
   small seeded problems into pins.json.

PETSc binary layout (big endian): Mat = int32 classid 1211216, M, N, nnz, row
lengths[M], column indices[nnz], float64 values[nnz]; Vec = int32 classid 1211214,
n, float64 values[n].
"""

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

MAT_ID, VEC_ID = 1211216, 1211214


def read_petsc(path):
    raw = open(path, "rb").read()
    cid = int(np.frombuffer(raw[:4], ">i4")[0])
    if cid == VEC_ID:
        n = int(np.frombuffer(raw[4:8], ">i4")[0])
        return np.frombuffer(raw[8:8 + 8 * n], ">f8").astype(np.float64)
    assert cid == MAT_ID, f"{path}: unknown PETSc class id {cid}"
    M, N, nz = (int(v) for v in np.frombuffer(raw[4:16], ">i4"))
    off = 16
    lens = np.frombuffer(raw[off:off + 4 * M], ">i4").astype(np.int64)
    off += 4 * M
    cols = np.frombuffer(raw[off:off + 4 * nz], ">i4").astype(np.int32)
    off += 4 * nz
    vals = np.frombuffer(raw[off:off + 8 * nz], ">f8").astype(np.float64)
    rp = np.zeros(M + 1, np.int64)
    np.cumsum(lens, out=rp[1:])
    # PETSc stores sorted columns per row; keep the order but check it
    for i in range(M):
        seg = cols[rp[i]:rp[i + 1]]
        assert np.all(np.diff(seg) > 0), "unsorted PETSc row"
    return {"shape": np.array([M, N]), "rowptr": rp.astype(np.int32), "colidx": cols, "values": vals}


def dump_mat(d, prefix, m):
    d[prefix + "_shape"] = m["shape"]
    d[prefix + "_rowptr"] = m["rowptr"]
    d[prefix + "_colidx"] = m["colidx"]
    d[prefix + "_values"] = m["values"]


def structure_digest(rp, ci):
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(rp, np.int32).tobytes())
    h.update(np.ascontiguousarray(ci, np.int32).tobytes())
    return h.hexdigest()


def main():
    if len(sys.argv) < 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the utopia reference checkout>")
    ref = sys.argv[1]
    base = os.path.join(ref, "utopia", "data")
    d = {}
    lap = os.path.join(base, "laplace", "matrices_for_petsc")
    dump_mat(d, "A", read_petsc(os.path.join(lap, "f_A")))
    d["rhs"] = read_petsc(os.path.join(lap, "f_rhs"))
    for k in (1, 2, 3):
        dump_mat(d, f"I{k}", read_petsc(os.path.join(lap, f"I_{k}")))
    np.savez_compressed(os.path.join(HERE, "laplace_hierarchy.npz"), **d)
    d = {}
    mg = os.path.join(base, "mg")
    dump_mat(d, "A", read_petsc(os.path.join(mg, "A.bin")))
    dump_mat(d, "I", read_petsc(os.path.join(mg, "I.bin")))
    d["rhs"] = read_petsc(os.path.join(mg, "rhs.bin"))
    np.savez_compressed(os.path.join(HERE, "mg_two_level.npz"), **d)

    # oracle regression pins
    import oracle as O
    from utopia_gb300 import problems as P
    pins = {}
    A, b = P.poisson2d_cg(64, seed=0)
    x, st = O.cg_solve(O.Matrix(A), b, atol=1e-8 * np.linalg.norm(b))
    pins["cg_jacobi_poisson2d_64"] = {"iterates": st["iterates"], "x_norm": float(np.linalg.norm(x))}
    A, Ps, b = P.poisson3d_mg(32, 3, seed=1)
    Am = O.Matrix(A)
    mg = O.Multigrid(Am, Ps, smoother="chebyshev", pre=3, post=3)
    pins["galerkin_poisson3d_32"] = {
        f"level{l}": structure_digest(*mg.level_matrix(l).arrays()[:2]) for l in range(mg.n_levels)}
    pins["galerkin_poisson3d_32"]["eigs"] = [mg.eigs(l) for l in range(1, mg.n_levels)]
    x, st = O.cg_solve(Am, b, precond="mg", mg=mg, atol=1e-10 * np.linalg.norm(b))
    pins["mgpcg_chebyshev_poisson3d_32"] = {"iterates": st["iterates"]}
    with open(os.path.join(HERE, "pins.json"), "w") as f:
        json.dump(pins, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
