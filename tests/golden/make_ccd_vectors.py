"""Golden vectors for the moving-point / moving-triangle CCD test — run in the
container that holds the reference tree.

Builds the reference's own test (CollisionDetector/CCDSolver.h with its CyCodeBase
headers) with `make -C oracle ref` into oracle/_ref/libccd_ref.so, evaluates it on
seeded FP32 configurations (a triangle near the point's path, moving or static, at
unit and centimetre scale) and stores inputs and outputs in ccd_vectors.npz next to
this script. tests/test_tet_contact_host.py checks the oracle's restatement against
them bit for bit.

    python tests/golden/make_ccd_vectors.py
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.join(HERE, "..", "..", "oracle")


def cases(n: int, seed: int = 11):
    rng = np.random.default_rng(seed)
    x0 = np.empty((n, 9), np.float32)
    x1 = np.empty((n, 9), np.float32)
    p0 = np.empty((n, 3), np.float32)
    p1 = np.empty((n, 3), np.float32)
    for k in range(n):
        mode = k % 5
        scale = 1e-2 if mode == 4 else 1.0
        base = rng.uniform(-1, 1, 3) * (0.5 if mode == 4 else 1.0)
        a = (base + rng.normal(0, scale, 9).reshape(3, 3)).astype(np.float32).ravel()
        if mode == 2:
            b = a.copy()
        elif mode == 3:
            b = (a.reshape(3, 3) + rng.normal(0, scale, 3)).astype(np.float32).ravel()
        else:
            b = (a + rng.normal(0, scale * 0.3, 9)).astype(np.float32)
        c0, c1 = a.reshape(3, 3).mean(0), b.reshape(3, 3).mean(0)
        nrm = np.cross(a[3:6] - a[0:3], a[6:9] - a[0:3])
        nrm /= np.linalg.norm(nrm) + 1e-30
        off = rng.normal(0, scale * 0.3, 3)
        x0[k], x1[k] = a, b
        p0[k] = (c0 + off + nrm * scale * 0.2).astype(np.float32)
        p1[k] = (c1 + off * rng.uniform(0.5, 1.5) - nrm * scale * 0.2).astype(np.float32)
    return x0, x1, p0, p1


def evaluate(fn, x0, x1, p0, p1):
    fp = C.POINTER(C.c_float)
    n = len(x0)
    hit = np.zeros(n, np.int32)
    tt = np.zeros(n, np.float32)
    bary = np.zeros((n, 3), np.float32)
    for k in range(n):
        t = np.zeros(1, np.float32)
        b = np.zeros(3, np.float32)
        args = [np.ascontiguousarray(v[k]) for v in (x0, x1, p0, p1)]
        hit[k] = fn(*[v.ctypes.data_as(fp) for v in args], t.ctypes.data_as(fp), b.ctypes.data_as(fp))
        tt[k] = t[0]
        bary[k] = b
    return hit, tt, bary


def main():
    subprocess.run(["make", "-s", "-C", ORACLE, "ref"], check=True)
    lib = C.CDLL(os.path.join(ORACLE, "_ref", "libccd_ref.so"))
    fn = lib.ref_ccd_tri_point
    fn.argtypes = [C.POINTER(C.c_float)] * 6
    fn.restype = C.c_int32
    x0, x1, p0, p1 = cases(2000)
    hit, tt, bary = evaluate(fn, x0, x1, p0, p1)
    np.savez_compressed(os.path.join(HERE, "ccd_vectors.npz"), x0=x0, x1=x1, p0=p0, p1=p1, hit=hit, tt=tt, bary=bary)
    print("cases", len(hit), "hits", int(hit.sum()))


if __name__ == "__main__":
    main()
