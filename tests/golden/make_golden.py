"""Writes the golden fixtures of tests/golden/ from the reference's own code.

Run in a checkout that has the reference sources (Pathlessbark8/C-_serial):

    QLSKUM_REFERENCE_DIR=/path/to/reference python tests/golden/make_golden.py

It compiles the reference through oracle/build_ref.sh (the unmodified
headers driven by oracle/ref_harness.cpp) and records, for seeded clouds from
qlskum.cloudgen:

* flux_kat.npz      -- the 8 split / quadrant fluxes of the reference
                       (split_fluxes_mod.h, quadrant_fluxes_mod.h) on rows of
                       the reference's own data.dat input fixture (columns
                       nx ny u1 u2 rho pr, as main.cpp:72-100 reads them);
* cloud_small.npz   -- a 480-point NACA 0012 cloud (40 wall points x 12 rings,
                       first spacing 1e-2, far field at 5 chords);
* ref_small_run.npz   -- 50 iterations at M 0.63, AoA 2, inner 0: residual
                       history, final prim, Cl / Cd / Cm / entropy;
* cloud_trans.npz     -- a 2,560-point cloud (64 x 40, far field at 3 chords;
                       the defect-correction inner loop needs a finer far
                       field than the 480-point cloud has to stay stable);
* ref_trans_stage.npz -- one dumped stage after 5 iterations (M 0.63,
                       inner 2): q, dq before / after the inner loop, qm,
                       delta, flux_res, prim before / after state_update(1),
                       the sub-stencils and normals;
* ref_trans_run.npz   -- 30 iterations at M 0.85, AoA 1, inner 3;
* cloud_c1.npz + ref_c1_run.npz -- the 9,600-point cloud (160 wall points x
                       60 rings) and 1000 reference iterations with the
                       plain FP64 recipe (M 0.63, AoA 2, CFL 0.2, VL 50,
                       power 0, inner 0).
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "c-_serial_gb300"))
sys.path.insert(0, os.path.join(REPO, "oracle"))

from qlskum import cloudgen  # noqa: E402
import qlskum_oracle  # noqa: E402

SMALL = dict(n_wall=40, n_layers=12, first_spacing=1e-2, radius=5.0, seed=7)
TRANS = dict(n_wall=64, n_layers=40, first_spacing=5e-3, radius=3.0, seed=11)


def cloud_arrays(c):
    return dict(x=c.x, y=c.y, left=c.left, right=c.right, flag_1=c.flag_1, flag_2=c.flag_2, min_dist=c.min_dist,
                nbhs=c.nbhs, conn=c.conn)


def run_ref(binary, mode, grid, **kw):
    out = tempfile.mkdtemp(prefix="qlskum_golden_")
    args = [binary, mode, grid, out] + [f"{k}={v}" for k, v in kw.items()]
    subprocess.check_call(args, cwd=out, stdout=subprocess.DEVNULL)
    res = {}
    for f in os.listdir(out):
        p = os.path.join(out, f)
        if f.endswith(".f64"):
            res[f[:-4]] = np.fromfile(p, np.float64)
        elif f.endswith(".i32"):
            res[f[:-4]] = np.fromfile(p, np.int32)
    return res


def main():
    ref = qlskum_oracle.build_reference()
    refdir = qlskum_oracle.reference_dir()
    if ref is None or refdir is None:
        sys.exit("reference sources not found (set QLSKUM_REFERENCE_DIR)")

    # flux KAT on data.dat rows
    rows = np.loadtxt(os.path.join(refdir, "data.dat"))[:400]
    tmp = tempfile.mkdtemp()
    np.savetxt(os.path.join(tmp, "rows.dat"), rows, fmt="%.17g")
    subprocess.check_call([ref, "flux", os.path.join(tmp, "rows.dat"), os.path.join(tmp, "flux.bin")])
    G = np.fromfile(os.path.join(tmp, "flux.bin")).reshape(-1, 8, 4)
    np.savez_compressed(os.path.join(HERE, "flux_kat.npz"), inputs=rows[:, 4:], outputs=G)

    # small cloud
    c = cloudgen.make_cloud(**SMALL)
    np.savez_compressed(os.path.join(HERE, "cloud_small.npz"), **cloud_arrays(c))
    grid = os.path.join(tmp, "small.grid")
    cloudgen.write_partgrid(c, grid)
    n = c.n
    r = run_ref(ref, "run", grid, mach=0.63, aoa=2, cfl=0.2, vl=50, inner=0, power=0, iters=50)
    np.savez_compressed(os.path.join(HERE, "ref_small_run.npz"), residuals=r["residuals"].reshape(-1, 3),
                        prim=r["prim"].reshape(n, 4), objectives=r["objectives"])
    ct = cloudgen.make_cloud(**TRANS)
    np.savez_compressed(os.path.join(HERE, "cloud_trans.npz"), **cloud_arrays(ct))
    gridt = os.path.join(tmp, "trans.grid")
    cloudgen.write_partgrid(ct, gridt)
    st = run_ref(ref, "stage", gridt, mach=0.63, aoa=2, cfl=0.2, vl=50, inner=2, power=0, iters=5)
    np.savez_compressed(
        os.path.join(HERE, "ref_trans_stage.npz"),
        prim_in=st["prim_in"].reshape(ct.n, 4), delta=st["delta"], q=st["q"].reshape(ct.n, 4),
        dq0=st["dq0"].reshape(ct.n, 2, 4), qm=st["qm"].reshape(ct.n, 2, 4), dq=st["dq"].reshape(ct.n, 2, 4),
        flux_res=st["flux_res"].reshape(ct.n, 4), prim_out=st["prim_out"].reshape(ct.n, 4), stage_res=st["stage_res"],
        sub_counts=st["sub_counts"].reshape(ct.n, 4), sub_lists=st["sub_lists"], normals=st["normals"].reshape(ct.n, 2),
        residuals=st["residuals"].reshape(-1, 3))
    r = run_ref(ref, "run", gridt, mach=0.85, aoa=1, cfl=0.2, vl=50, inner=3, power=0, iters=30)
    np.savez_compressed(os.path.join(HERE, "ref_trans_run.npz"), residuals=r["residuals"].reshape(-1, 3),
                        prim=r["prim"].reshape(ct.n, 4), objectives=r["objectives"])

    if "--no-c1" in sys.argv:  # keep the existing config-1 fixtures (4 minutes of reference time)
        print("golden fixtures written to", HERE)
        return
    # config-1 cloud, 1000 iterations
    c1 = cloudgen.config1_cloud()
    np.savez_compressed(os.path.join(HERE, "cloud_c1.npz"), **cloud_arrays(c1))
    grid1 = os.path.join(tmp, "c1.grid")
    cloudgen.write_partgrid(c1, grid1)
    r = run_ref(ref, "run", grid1, mach=0.63, aoa=2, cfl=0.2, vl=50, inner=0, power=0, iters=1000)
    np.savez_compressed(os.path.join(HERE, "ref_c1_run.npz"), residuals=r["residuals"].reshape(-1, 3),
                        prim=r["prim"].reshape(c1.n, 4), objectives=r["objectives"],
                        sub_counts=r["sub_counts"].reshape(c1.n, 4))
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
