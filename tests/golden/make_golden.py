"""Generate the golden fixtures under tests/golden/ by running the UNMODIFIED
reference (UW-OCP/Collocation-Solver-CUDA) on the CPU.

The reference is Python + numba-CUDA.  numba and a GPU are absent here, so
``refshim/`` supplies a CPU stand-in for the few numba.cuda calls it makes
(kernels run thread by thread; see refshim/numba/__init__.py).  The reference
sources are imported read-only from REF_DIR; nothing is copied.

Outputs (all small, committed):

* ``e2e_<case>.npz``   : full solve via ``collocation_solver_parallel(m)``:
  Newton norm sequence, counts from the reference's benchmark file, final mesh
  size, maximum segment residual and the written solution file (t, y, z, p).
* ``stage_<case>.npz`` : one call of every stage function on a seeded random
  state: residual, Jacobian blocks, condensation, partitioned BABD solve,
  recovery, segment residual, node recovery, remesh, initial input.
* ``segres_<case>.npz``: the segment residual of a stage dump's state under
  every estimate the reference offers (residual_type 0/1/2 with and without
  scale_by_time, and residual2).
* ``e2e_vdp_coarse_res2.npz``: an end-to-end solve with residual2 on.
* ``fe_<case>.npz``    : the generated problem functions f, g, r, Df, Dg, Dr
  evaluated at seeded random points, plus the generated BvpDae attributes.
* the OCP sources used are in ``ocp/``.

Usage:  REF_DIR=<reference checkout> python tests/golden/make_golden.py [case ...]
Needs the reference checkout (read-only) and sympy; runs in a few minutes.
"""
import json
import os
import re
import shutil
import subprocess
import sys
import tempfile

import numpy as np

REF_DIR = os.environ.get("REF_DIR")
if not REF_DIR and __name__ == "__main__":
    sys.exit("set REF_DIR to the reference checkout (read-only), e.g. REF_DIR=/root/reference")
HERE = os.path.dirname(os.path.abspath(__file__))
SHIM = os.path.join(HERE, "refshim")
OCP_DIR = os.path.join(HERE, "ocp")

# (case name, ocp file, m) for end-to-end solves
E2E_CASES = [
    ("vdp_cfg1", "vdp.ocp", 4),
    ("vdp_coarse", "vdp_coarse.ocp", 3),
    ("dint_param", "dint_param.ocp", 3),
    ("pend2", "pend2.ocp", 4),
    ("vdp_ineq", "vdp_ineq.ocp", 3),
    ("vdp_input", "vdp_input.ocp", 4),
    ("vdp_svineq", "vdp_svineq.ocp", 3),
    ("vdp_m7", "vdp.ocp", 7),
    ("eqcon", "eqcon.ocp", 3),
]
# (case name, ocp file, m, N nodes, seed) for per-stage dumps
STAGE_CASES = [
    ("vdp_n21_m4", "vdp.ocp", 4, 21, 11),
    ("vdp_n33_m5", "vdp.ocp", 5, 33, 12),
    ("dint_n33_m3", "dint_param.ocp", 3, 33, 13),
    ("pend2_n21_m5", "pend2.ocp", 5, 21, 14),
    ("econ_n17_m3", "eqcon.ocp", 3, 17, 15),
]
# front-end cases: every OCP file in ocp/ plus the reference notebook sources
NOTEBOOK_OCPS = ["exContainerTransfer", "exFreespaceRocket", "exTrolley", "exUnderwaterVehicle"]


def _env():
    env = dict(os.environ)
    env["PYTHONPATH"] = os.pathsep.join([SHIM, REF_DIR])
    return env


def _copy_inputs(workdir):
    """Solution files that OCPs name as InputFile."""
    for fn in os.listdir(OCP_DIR):
        if fn.endswith(".data"):
            shutil.copy(os.path.join(OCP_DIR, fn), workdir)


def _gen_problem(ocp_path, workdir):
    """Run the reference's OCP2ABVP.py on an OCP file -> bvp_problem.py in workdir."""
    out = subprocess.run([sys.executable, os.path.join(REF_DIR, "OCP2ABVP.py"), ocp_path],
                         cwd=workdir, env=_env(), capture_output=True, text=True, check=True)
    with open(os.path.join(workdir, "bvp_problem.py"), "w") as f:
        f.write(out.stdout)


# ----------------------------------------------------------------- e2e ------
def run_e2e(case, ocp_file, m, driver=None):
    """driver: source of a script taking m that runs the reference driver
    (default: the reference's own command line)."""
    work = tempfile.mkdtemp(prefix="golden_e2e_")
    try:
        shutil.copy(os.path.join(OCP_DIR, ocp_file), work)
        _copy_inputs(work)
        _gen_problem(ocp_file, work)
        env = _env()
        env["PYTHONPATH"] = os.pathsep.join([work, SHIM, REF_DIR])
        if driver is None:
            cmd = [sys.executable, os.path.join(REF_DIR, "collocation_solver_parallel_2d_shared.py"), "-m", str(m)]
        else:
            with open(os.path.join(work, "driver.py"), "w") as f:
                f.write(driver)
            cmd = [sys.executable, "driver.py", str(m)]
        p = subprocess.run(cmd, cwd=work, env=env, capture_output=True, text=True, timeout=7200)
        log = p.stdout
        if p.returncode != 0:
            raise RuntimeError(p.stderr[-3000:])
        norms = [float(x) for x in re.findall(r"norm: ([0-9.eE+-]+)", log)]
        nodes_after = [int(x) for x in re.findall(r"Remeshed the problem. Number of nodes = (\d+)", log)]
        alphas = [float(x) for x in re.findall(r"Continuation iteration: \d+, solving alpha = ([0-9.eE+-]+)", log)]
        max_res = float(re.findall(r"Maximum residual: ([0-9.eE+-]+)", log)[-1])
        success = "Problem solved successfully." in log
        bench = {}
        bdir = os.path.join(work, "benchmark_performance")
        for fn in os.listdir(bdir):
            for line in open(os.path.join(bdir, fn)):
                k, v = line.split(":")
                if "counts" in k:
                    bench[k.strip()] = int(v)
        sys.path.insert(0, REF_DIR)
        from BVPDAEReadWriteData import bvpdae_read_data  # noqa: E402  (reference reader)
        outname = re.search(r"self.output_file = '([^']+)'", open(os.path.join(work, "bvp_problem.py")).read()).group(1)
        err, t, y, z, pp = bvpdae_read_data(os.path.join(work, outname))
        assert err == 0
        np.savez_compressed(os.path.join(HERE, "e2e_%s.npz" % case),
                 m=m, norms=np.array(norms), nodes_after_remesh=np.array(nodes_after, dtype=np.int64),
                 alphas=np.array(alphas), max_residual=max_res, success=success,
                 residual_counts=bench.get("Residual counts", -1), jacobian_counts=bench.get("Jacobian counts", -1),
                 segment_counts=bench.get("Segment Residual counts", -1),
                 t=np.asarray(t), y=np.asarray(y), z=np.asarray(z), p=np.asarray(pp),
                 output_text=open(os.path.join(work, outname)).read(), log=log)
        print("e2e %s: %d norms, final N=%d, maxres=%g, success=%s" % (case, len(norms), len(t), max_res, success))
    finally:
        shutil.rmtree(work, ignore_errors=True)


# --------------------------------------------------------------- stages -----
STAGE_SCRIPT = r'''
import sys, json
import numpy as np
case, m, N, seed, out = sys.argv[1], int(sys.argv[2]), int(sys.argv[3]), int(sys.argv[4]), sys.argv[5]
import collocation_solver_parallel_2d_shared as CS
import solve_babd_system as SB
import collocation_coefficients
import bvp_problem
bd = bvp_problem.BvpDae()
ny, nz, np_ = bd.size_y, bd.size_z, bd.size_p
# module globals the reference sets inside collocation_solver_parallel()
CS.global_size_y, CS.global_size_z, CS.global_size_p = ny, nz, np_
CS.m_collocation = m
from math import ceil, log
CS.TPB_m = max(int(pow(2, ceil(log(m, 2)))), 2)
CS.global_y_shared_size = CS.TPB_N * m
rk = collocation_coefficients.lobatto(m)
rng = np.random.default_rng(seed)
t = np.sort(rng.uniform(0.0, 1.0, N)); t[0] = 0.0; t[-1] = 1.0
t = t * bd.t_final if hasattr(bd, "t_final") else t
y0 = 0.3 * rng.standard_normal((N, ny))
z0 = 0.3 * rng.standard_normal((N, nz))
p = 0.5 + 0.3 * rng.random(np_)
alpha = 0.1
d = {}
d["t"], d["y0"], d["z0"], d["p"] = t, y0, z0, p
y, y_dot, z_tilde = CS.form_initial_input_parallel(ny, nz, np_, m, N, y0, z0, p, rk)
d["init_y_dot"], d["init_z_tilde"] = y_dot, z_tilde
# perturb the stage values so that the residual is not trivially structured
y_dot = y_dot + 0.1 * rng.standard_normal(y_dot.shape)
z_tilde = z_tilde + 0.1 * rng.standard_normal(z_tilde.shape)
d["y"], d["y_dot"], d["z_tilde"] = y, y_dot, z_tilde
f_q, y_tilde, f_a, f_b, r_bc = CS.compute_f_q_parallel(ny, nz, np_, m, N, rk, t, y, y_dot, z_tilde, p, alpha)
d.update(f_q=f_q, y_tilde=y_tilde, f_a=f_a, f_b=f_b, r_bc=r_bc)
J, V, D, W, B_0, B_n, V_n = CS.construct_jacobian_parallel(ny, nz, np_, m, N, rk, t, y, y_tilde, z_tilde, p, alpha)
d.update(J=J, V=V, D=D, W=W, B_0=B_0, B_n=B_n, V_n=V_n)
A, C, H, b = CS.reduce_jacobian_parallel(ny, nz, np_, m, N, W, D, J, V, f_a, f_b)
d.update(A=A, C=C, H=H, b=b)
M = 8
index, R, E, J_red, G, dd, A_t, C_t, H_t, b_t = SB.partition_factorization_parallel(ny, np_, M, N, A, C, H, b)
d.update(index=index, R=R, E=E, J_red=J_red, G=G, d=dd, A_tilde=A_t, C_tilde=C_t, H_tilde=H_t, b_tilde=b_t)
sol = SB.construct_babd_mshoot(ny, 0, np_, M, A_t, C_t, H_t, b_t, B_0, B_n, V_n, -r_bc)
SB.qr_decomposition(ny, np_, M + 1, sol)
SB.backward_substitution(M + 1, sol)
delta_s_r, delta_p = SB.recover_babd_solution(M, ny, 0, np_, sol)
delta_y = SB.partition_backward_substitution_parallel(ny, np_, M, N, index, delta_s_r, delta_p, R, G, E, J_red, dd)
d.update(delta_s_r=delta_s_r, delta_p=delta_p, delta_y=delta_y)
delta_k, delta_y_dot, delta_z_tilde = CS.recover_delta_k_parallel(ny, nz, m, N, delta_y, delta_p, f_a, J, V, W)
d.update(delta_k=delta_k, delta_y_dot=delta_y_dot, delta_z_tilde=delta_z_tilde)
tol = 1e-6
residual, max_residual = CS.compute_segment_residual_parallel(ny, nz, np_, m, N, t, y, y_dot, z_tilde, p, alpha, tol)
d.update(seg_residual=residual, seg_max=max_residual)
z_nodes = CS.recover_solution_parallel(nz, m, N, z_tilde)
d["z_nodes"] = z_nodes
# remesh on a synthetic residual that exercises deletion, midpoint and 3-point insertion
res = np.exp(rng.uniform(np.log(1e-4), np.log(100.0), N))
res[2:9] = 1e-3
res[-7:] = 1e-3
d["remesh_residual"] = res
N_new, t_new, y_new, z_new = CS.remesh(ny, nz, N, t, y, z_nodes, res)
d.update(remesh_N=N_new, remesh_t=t_new, remesh_y=y_new, remesh_z=z_new)
np.savez_compressed(out, m=m, N=N, ny=ny, nz=nz, np=np_, alpha=alpha, tol=tol, **d)
print("stage", case, "ok")
'''


def run_stage(case, ocp_file, m, N, seed):
    work = tempfile.mkdtemp(prefix="golden_stage_")
    try:
        shutil.copy(os.path.join(OCP_DIR, ocp_file), work)
        _gen_problem(ocp_file, work)
        with open(os.path.join(work, "stage_dump.py"), "w") as f:
            f.write(STAGE_SCRIPT)
        env = _env()
        env["PYTHONPATH"] = os.pathsep.join([work, SHIM, REF_DIR])
        out = os.path.join(HERE, "stage_%s.npz" % case)
        p = subprocess.run([sys.executable, "stage_dump.py", case, str(m), str(N), str(seed), out],
                           cwd=work, env=env, capture_output=True, text=True, timeout=3600)
        if p.returncode != 0:
            raise RuntimeError(p.stderr[-3000:])
        print(p.stdout.strip().splitlines()[-1])
    finally:
        shutil.rmtree(work, ignore_errors=True)


# ------------------------------------------------- segment residual modes ---
# The reference's estimate is switched by module globals (residual_type 0/1/2,
# scale_by_time, residual2; collocation_solver_parallel_2d_shared.py:29-32,
# 1770-2013).  On the state of a stage dump, record every combination.
SEGRES_SCRIPT = r'''
import sys
import numpy as np
stage, out = sys.argv[1], sys.argv[2]
import collocation_solver_parallel_2d_shared as CS
import bvp_problem
g = np.load(stage)
bd = bvp_problem.BvpDae()
ny, nz, np_ = bd.size_y, bd.size_z, bd.size_p
m, N = int(g["m"]), int(g["N"])
CS.global_size_y, CS.global_size_z, CS.global_size_p = ny, nz, np_
CS.m_collocation = m
args = (ny, nz, np_, m, N, g["t"], g["y"], g["y_dot"], g["z_tilde"], g["p"], float(g["alpha"]), float(g["tol"]))
d = {}
for rt in (0, 1, 2):
    for sc in (True, False):
        CS.residual_type, CS.scale_by_time = rt, sc
        res, mx = CS.compute_segment_residual_parallel(*args)
        d["res_t%d_s%d" % (rt, int(sc))] = res
        d["max_t%d_s%d" % (rt, int(sc))] = mx
res, mx = CS.compute_segment_residual_parallel2(*args)
d["res2"], d["max2"] = res, mx
np.savez_compressed(out, **d)
print("segres ok")
'''


def run_segres(case, ocp_file):
    work = tempfile.mkdtemp(prefix="golden_segres_")
    try:
        shutil.copy(os.path.join(OCP_DIR, ocp_file), work)
        _gen_problem(ocp_file, work)
        with open(os.path.join(work, "segres_dump.py"), "w") as f:
            f.write(SEGRES_SCRIPT)
        env = _env()
        env["PYTHONPATH"] = os.pathsep.join([work, SHIM, REF_DIR])
        p = subprocess.run([sys.executable, "segres_dump.py", os.path.join(HERE, "stage_%s.npz" % case),
                            os.path.join(HERE, "segres_%s.npz" % case)], cwd=work, env=env, capture_output=True,
                           text=True, timeout=3600)
        if p.returncode != 0:
            raise RuntimeError(p.stderr[-3000:])
        print(case, p.stdout.strip().splitlines()[-1])
    finally:
        shutil.rmtree(work, ignore_errors=True)


# e2e solves with the residual2 estimate (module global set before the driver)
RES2_SCRIPT = r'''
import sys
import collocation_solver_parallel_2d_shared as CS
CS.residual2 = True
CS.collocation_solver_parallel(m=int(sys.argv[1]))
'''
E2E_RES2_CASES = [("vdp_coarse_res2", "vdp_coarse.ocp", 3)]


# ------------------------------------------------------------ front end -----
FE_SCRIPT = r'''
import sys
import numpy as np
out, seed = sys.argv[1], int(sys.argv[2])
import bvp_problem as bp
try:
    bd = bp.BvpDae()
except Exception:
    bd = None
attrs = {}
ny = nz = np_ = None
src = open("bvp_problem.py").read()
import re
ny = int(re.search(r"self.size_y = (\d+)", src).group(1))
nz = int(re.search(r"self.size_z = (\d+)", src).group(1))
np_ = int(re.search(r"self.size_p = (\d+)", src).group(1))
nineq = int(re.search(r"self.size_inequality = (\d+)", src).group(1))
nsv = int(re.search(r"self.size_sv_inequality = (\d+)", src).group(1))
rng = np.random.default_rng(seed)
K = 8
Y = 0.5 + 0.4 * rng.random((K, ny)); Z = 0.5 + 0.4 * rng.random((K, nz)); P = 0.5 + 0.4 * rng.random((K, np_))
Y1 = 0.5 + 0.4 * rng.random((K, ny)); AL = 0.01 + 0.1 * rng.random(K)
F = np.zeros((K, ny)); G = np.zeros((K, nz)); R = np.zeros((K, ny + np_))
DF = np.zeros((K, ny, ny + nz + np_)); DG = np.zeros((K, nz, ny + nz + np_)); DR = np.zeros((K, ny + np_, 2 * ny + np_))
for k in range(K):
    bp._abvp_f(Y[k], Z[k], P[k], F[k])
    bp._abvp_g(Y[k], Z[k], P[k], AL[k], G[k])
    bp._abvp_r(Y[k], Y1[k], P[k], R[k])
    bp._abvp_Df(Y[k], Z[k], P[k], DF[k])
    bp._abvp_Dg(Y[k], Z[k], P[k], AL[k], DG[k])
    bp._abvp_Dr(Y[k], Y1[k], P[k], DR[k])
extra = {}
if bd is not None:
    extra = dict(T0=bd.T0, Y0=bd.Y0, Z0=bd.Z0, P0=bd.P0, tolerance=bd.tolerance,
                 maximum_nodes=bd.maximum_nodes, maximum_newton_iterations=bd.maximum_newton_iterations,
                 maximum_mesh_refinements=bd.maximum_mesh_refinements, output_file=bd.output_file)
np.savez_compressed(out, ny=ny, nz=nz, np=np_, n_ineq=nineq, n_svineq=nsv, Y=Y, Z=Z, P=P, Y1=Y1, ALPHA=AL,
         F=F, G=G, R=R, DF=DF, DG=DG, DR=DR, has_bvpdae=bd is not None, **extra)
print("fe ok", ny, nz, np_)
'''


def run_fe(case, ocp_path, seed):
    work = tempfile.mkdtemp(prefix="golden_fe_")
    try:
        shutil.copy(ocp_path, work)
        _copy_inputs(work)
        _gen_problem(os.path.basename(ocp_path), work)
        with open(os.path.join(work, "fe_dump.py"), "w") as f:
            f.write(FE_SCRIPT)
        env = _env()
        env["PYTHONPATH"] = os.pathsep.join([work, SHIM, REF_DIR])
        out = os.path.join(HERE, "fe_%s.npz" % case)
        p = subprocess.run([sys.executable, "fe_dump.py", out, str(seed)], cwd=work, env=env,
                           capture_output=True, text=True, timeout=600)
        if p.returncode != 0:
            raise RuntimeError(p.stderr[-3000:])
        print("fe", case, p.stdout.strip().splitlines()[-1])
    finally:
        shutil.rmtree(work, ignore_errors=True)


TABLES_SCRIPT = r'''
import sys
import numpy as np
import collocation_coefficients as CC
import gauss_coefficients as GC
d = {}
for m in range(3, 11):
    r = CC.lobatto(m)
    d["A%d" % m], d["b%d" % m], d["c%d" % m] = r.A, r.b, r.c
    g = GC.gauss(m + 1)
    L = np.zeros((m + 1, m)); I = np.zeros((m + 1, m)); l = np.zeros(m)
    for i, tau in enumerate(g.t):
        CC.compute_L(m, tau, l); L[i] = l
        CC.compute_I(m, tau, l); I[i] = l
    d["L%d" % m], d["I%d" % m] = L, I
for n in range(2, 12):
    g = GC.gauss(n)
    d["gt%d" % n], d["gw%d" % n] = g.t, g.w
np.savez_compressed(sys.argv[1], **d)
print("tables ok")
'''


def run_tables():
    work = tempfile.mkdtemp(prefix="golden_tab_")
    try:
        with open(os.path.join(work, "tab.py"), "w") as f:
            f.write(TABLES_SCRIPT)
        p = subprocess.run([sys.executable, "tab.py", os.path.join(HERE, "tables.npz")], cwd=work, env=_env(),
                           capture_output=True, text=True, timeout=600)
        if p.returncode != 0:
            raise RuntimeError(p.stderr[-3000:])
        print(p.stdout.strip())
    finally:
        shutil.rmtree(work, ignore_errors=True)


def main(argv):
    want = set(argv)
    sel = (lambda name: not want or name in want)
    if sel("tables"):
        run_tables()
    for i, f in enumerate(sorted(x for x in os.listdir(OCP_DIR) if x.endswith(".ocp"))):
        name = os.path.splitext(f)[0]
        if sel("fe_" + name):
            run_fe(name, os.path.join(OCP_DIR, f), 100 + i)
    for i, nb in enumerate(NOTEBOOK_OCPS):
        if sel("fe_" + nb):
            run_fe(nb, os.path.join(REF_DIR, "Notebook", "source", nb), 200 + i)
    for case in STAGE_CASES:
        if sel("stage_" + case[0]):
            run_stage(*case)
    for case in STAGE_CASES:
        if sel("segres_" + case[0]):
            run_segres(case[0], case[1])
    for case in E2E_CASES:
        if sel("e2e_" + case[0]):
            run_e2e(*case)
    for case in E2E_RES2_CASES:
        if sel("e2e_" + case[0]):
            run_e2e(*case, driver=RES2_SCRIPT)


if __name__ == "__main__":
    main(sys.argv[1:])
