"""Generate the committed golden fixtures from the reference implementation.

Run here, where the reference tree exists (it is not needed anywhere else):

    python tests/golden/make_golden.py

Steps: build oracle/_ref/ref_harness from the reference headers (oracle/Makefile,
target `ref`), write each synthetic system as Matrix Market plus a raw FP64 right-
hand side, run the harness (which reads the matrix with the reference's own
io::ReadMM, applies LMax1Scaling, builds the reference's FP64/FP32/int AMG
preconditioners and solvers and dumps their arrays and kernel input/output pairs),
and pack every dumped array into tests/golden/<case>.npz together with the
harness's stdout.
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
import gen_matrices as gm  # noqa: E402

HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")

# name: (generator, smoother 0=SOR 1=BlockSOR-40 2=JacobiSOR, m, what, dump_cycle)
CASES = {
    "p2d64": (lambda: gm.poisson2d(64), 0, 30, "fp64,fp32,inth,ints,dh", 1),
    "p3d16": (lambda: gm.poisson3d(16), 0, 30, "fp64,fp32,inth,ints,dh,fh", 1),
    "cd3d16": (lambda: gm.convdiff3d(16, 50.0), 0, 30, "fp64,fp32,inth,ints", 1),
    "vc3d16": (lambda: gm.varcoef3d(16, 2.0, 7), 0, 30, "fp64,fp32,inth,ints", 0),
    # the reference's int solve overflows int32 on this system with the rule's
    # bit (blas1.hpp:43, then a division by zero at gmres.hpp:244), so only its
    # int hierarchy and kernels are recorded
    "an2d64": (lambda: gm.aniso2d(64, 1e-3), 0, 30, "fp64,fp32,inth", 0),
    "s27n14": (lambda: gm.stencil27(14, 11), 0, 20, "fp64,fp32,inth,ints", 0),
    "p3d16bj": (lambda: gm.poisson3d(16), 1, 30, "fp64,inth,ints", 0),
    # JacobiSORflex: 1200-row chunks (4 on the finest level of both systems)
    "p3d16js": (lambda: gm.poisson3d(16), 2, 30, "fp64,inth,ints", 0),
    "p2d64js": (lambda: gm.poisson2d(64), 2, 30, "fp64,inth,ints", 0),
}
RHS_SEED = 12345


def load_dir(d):
    out = {}
    for fn in sorted(os.listdir(d)):
        name, suf = fn.rsplit(".", 1)
        dt = {"i32": np.int32, "i64": np.int64, "f64": np.float64, "f32": np.float32}[suf]
        out[name] = np.fromfile(os.path.join(d, fn), dtype=dt)
    return out


def main():
    subprocess.check_call(["make", "-C", os.path.join(ROOT, "oracle"), "ref"])
    only = set(sys.argv[1:])
    with tempfile.TemporaryDirectory() as tmp:
        if not only or "blas" in only:
            od = os.path.join(tmp, "blas")
            os.makedirs(od)
            subprocess.check_call([HARNESS, "blas", od])
            np.savez_compressed(os.path.join(HERE, "blas.npz"), **load_dir(od))
            print("blas done")
        for name, (gen, smo, m, what, cyc) in CASES.items():
            if only and name not in only:
                continue
            rptr, cind, val = gen()
            xs, b = gm.rhs(rptr, cind, val, RHS_SEED)
            mtx = os.path.join(tmp, name + ".mtx")
            gm.write_mtx(mtx, rptr, cind, val)
            bpath = os.path.join(tmp, name + ".b")
            b.astype(np.float64).tofile(bpath)
            od = os.path.join(tmp, name)
            os.makedirs(od)
            res = subprocess.run([HARNESS, "solve", mtx, bpath, od, str(smo), str(m), what, str(cyc)],
                                 capture_output=True, text=True, check=True)
            arrays = load_dir(od)
            arrays["in_rptr"], arrays["in_cind"], arrays["in_val"] = rptr, cind, val
            arrays["in_b"] = b
            arrays["in_xstar"] = xs
            arrays["cfg"] = np.array([smo, m, cyc], dtype=np.int64)
            arrays["stdout"] = np.frombuffer(res.stdout.encode(), dtype=np.uint8)
            np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrays)
            iters = {k: int(arrays[k][0]) for k in ("int_iter", "fp64_iter", "fp32_iter") if k in arrays}
            print(name, "N=%d" % (len(rptr) - 1), "depth=%d" % int(arrays["depth"][0]) if "depth" in arrays else "",
                  "bit=%d" % int(arrays["bit"][0]), iters,
                  {k: float(arrays[k][0]) for k in ("int_res", "fp64_res", "fp32_res") if k in arrays})


if __name__ == "__main__":
    main()
