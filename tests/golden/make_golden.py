"""Generate golden vectors by running the reference's own C paths, compiled
from its sources by ``make -C oracle ref`` into oracle/_ref/: the steady-
transport solve (libfemref.so, oracle/ref_harness.c), the multi-dof EBE
operators (libfemref_*_blk.so, oracle/ref_block_harness.c), the 2D Euler
build and predictor (libfemref_euler.so, oracle/ref_euler_harness.c) and the
steady Navier-Stokes VMS build and damped Newton (libfemref_ns.so,
oracle/ref_ns_harness.c), the double-pairwise AMG preconditioner
(libfemref_amg.so, oracle/ref_amg_harness.c) and the transient transport
builds and Predictor_Old (libfemref_transient.so,
oracle/ref_transient_harness.c).

Usage:  python tests/golden/make_golden.py [case ...]   (writes tests/golden/*.npz;
        with case names, only those steady-transport cases)

The fixtures hold the inputs (mesh, node types, coefficient arrays evaluated by
the reference's plug-in callbacks) and every output the harness dumps: CSR
pattern, CSR_by_Element, node renumbering, EDE edge list, the first Build's
matrix storage and RHS, F after precond_setup, one matvec and one precond
application on a seeded vector, u after each Picard solve and the GMRES
iteration counts.  Only this script reads the reference library; the tests
read the committed .npz files.
"""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from fem_codes_gb300.mesh import structured_mesh  # noqa: E402

PROBLEMS = {"SKEW": 0, "CONVECTION": 1, "REACTION": 2, "HEMKER": 3, "VALIDACAO": 4}

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


def load_ref(fast: bool = False) -> ctypes.CDLL:
    name = "libfemref_fast.so" if fast else "libfemref.so"
    lib = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", name))
    f = lib.ref_transport_run
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, _dp, _dp, _ip, ctypes.c_int, _ip, ctypes.c_int,
                  ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p,
                  ctypes.c_char_p, ctypes.c_char_p,
                  ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_double,
                  _ip, _ip, _ip, _dp, _dp, _dp,
                  _ip, _ip, _ip, _ip,
                  _dp, _dp, _dp, _dp, _dp, _dp, _dp, _ip]
    return lib


def node_types(mesh, rule: str) -> np.ndarray:
    if rule == "inflow":      # x == 0 or y == 0 prescribed
        presc = (mesh.x == 0.0) | (mesh.y == 0.0)
    elif rule == "all":       # whole boundary prescribed
        presc = (mesh.x == 0.0) | (mesh.y == 0.0) | (mesh.x == 1.0) | (mesh.y == 1.0)
    else:
        raise ValueError(rule)
    return np.where(presc, 0, 1).astype(np.int32)


def run_ref(lib, mesh, ntype, problem="SKEW", scheme="CSR", reord="NOT", precond="ILU0",
            shock="CAU", hshock="2sqrtArea", outflow="NOT", kmax=30, lmax=1000,
            tol=1e-8, npicard=3, nonlin_tol=0.0, seed=7):
    nn, ne = mesh.nnodes, mesh.nel
    neq_ub = int((ntype >= 1).sum())
    nnz_ub = 9 * ne + 1
    info = np.zeros(5, np.int32)
    node_id = np.zeros(nn, np.int32)
    etype = np.zeros(ne, np.int32)
    beta = np.zeros(2 * ne)
    fsrc = np.zeros(3 * ne)
    upresc = np.zeros(nn)
    IA = np.zeros(neq_ub + 1, np.int32)
    JA = np.zeros(max(nnz_ub, 6 * ne + 2), np.int32)
    sbe = np.zeros(9 * ne, np.int32)
    order = np.zeros(3 * ne, np.int32)
    Afirst = np.zeros(max(9 * ne, 4 * (3 * ne + 1), nnz_ub))
    Ffirst = np.zeros(neq_ub + 1)
    Fprec = np.zeros(neq_ub + 1)
    rng = np.random.default_rng(seed)
    Pin = rng.uniform(-1.0, 1.0, neq_ub + 1)
    Qmv = np.zeros(neq_ub + 1)
    Zpc = np.zeros(neq_ub + 1)
    uhist = np.zeros(npicard * (neq_ub + 1))
    iters = np.zeros(npicard, np.int32)
    nit = lib.ref_transport_run(
        nn, np.ascontiguousarray(mesh.x), np.ascontiguousarray(mesh.y), ntype, ne,
        np.ascontiguousarray(mesh.vert.reshape(-1)), PROBLEMS[problem],
        scheme.encode(), reord.encode(), precond.encode(), shock.encode(), hshock.encode(),
        outflow.encode(), kmax, lmax, tol, npicard, nonlin_tol,
        info, node_id, etype, beta, fsrc, upresc, IA, JA, sbe, order,
        Afirst, Ffirst, Fprec, Pin, Qmv, Zpc, uhist, iters)
    neq, nnz, nedge, bw = (int(v) for v in info)
    out = dict(neq=neq, nnzero=nnz, nedge=nedge, bandwidth=bw, npicard_run=nit,
               node_id=node_id, etype=etype, beta=beta.reshape(ne, 2),
               fsrc=fsrc.reshape(ne, 3), upresc=upresc,
               Ffirst=Ffirst, Fprec=Fprec, Pin=Pin, Qmv=Qmv, Zpc=Zpc,
               uhist=uhist[: nit * (neq + 1)].reshape(nit, neq + 1), iters=iters[:nit])
    if scheme == "CSR":
        out.update(IA=IA[: neq + 1], JA=JA[:nnz], sbe=sbe.reshape(ne, 9), Afirst=Afirst[: nnz + 1])
    elif scheme == "EDE":
        out.update(lm2=JA[: 2 * nedge].reshape(nedge, 2), sbe=sbe[: 3 * ne].reshape(ne, 3),
                   order=order.reshape(ne, 3), Afirst=Afirst[: 4 * (nedge + 1)].reshape(nedge + 1, 4))
    else:
        out.update(Afirst=Afirst[: 9 * ne].reshape(ne, 9))
    return out


# name -> (nx, ny, perturb, node rule, run kwargs)
CASES = {
    "skew16_csr_ilu0_not": (16, 16, 0.0, "inflow", dict(scheme="CSR", reord="NOT", precond="ILU0")),
    "skew16_csr_ilu0_rcm": (16, 16, 0.2, "inflow", dict(scheme="CSR", reord="SYMRCM", precond="ILU0")),
    "skew16_ebe_none": (16, 16, 0.2, "inflow", dict(scheme="EBE", precond="NOT", npicard=2)),
    "skew16_ede_none": (16, 16, 0.2, "inflow", dict(scheme="EDE", precond="NOT", npicard=2)),
    "skew16_ebe_diag": (16, 16, 0.0, "inflow", dict(scheme="EBE", precond="Diag", npicard=2)),
    "skew24x12_csr_diag_yz": (24, 12, 0.2, "inflow", dict(scheme="CSR", precond="Diag", shock="YZBeta",
                                                          hshock="Option1", npicard=2)),
    "skew64_csr_ilu0_rcm": (64, 64, 0.0, "inflow", dict(scheme="CSR", reord="SYMRCM", precond="ILU0",
                                                       npicard=4)),
    "skew64_csr_ilu0_not": (64, 64, 0.0, "inflow", dict(scheme="CSR", reord="NOT", precond="ILU0",
                                                       npicard=2)),
    "reaction16_csr_ilu0": (16, 16, 0.1, "all", dict(problem="REACTION", scheme="CSR", precond="ILU0",
                                                     hshock="Option2", npicard=2)),
    "convection20_csr_rcm": (20, 20, 0.0, "inflow", dict(problem="CONVECTION", scheme="CSR", reord="SYMRCM",
                                                         precond="ILU0", hshock="sqrtArea",
                                                         outflow="YES", npicard=2)),
    "validacao16_ebe_diag": (16, 16, 0.15, "all", dict(problem="VALIDACAO", scheme="EBE", precond="Diag",
                                                       npicard=1)),
    "hemker12_ede_diag": (12, 12, 0.0, "inflow", dict(problem="HEMKER", scheme="EDE", precond="Diag",
                                                      npicard=1)),
    # ILU(p) with fill: "ILU1" / "ILU2" (ILUp_precond_setup.c:15, LEVEL_OF_FILL_lu)
    "skew16_csr_ilu1_rcm": (16, 16, 0.2, "inflow", dict(scheme="CSR", reord="SYMRCM", precond="ILU1", npicard=2)),
    "skew24x12_csr_ilu2": (24, 12, 0.1, "inflow", dict(scheme="CSR", reord="NOT", precond="ILU2", npicard=2)),
    # the plain-method configuration itself: 64x64 cells, CSR, ILU(0)-GMRES(30)
    # to 1e-8 (1000 restarts), the Picard loop run to its cap of 51 iterations
    # (Process.c:34; the iteration stagnates near max|du| = 0.04)
    "c1_skew64_csr_ilu0_51": (64, 64, 0.0, "inflow", dict(scheme="CSR", reord="NOT", precond="ILU0", kmax=30,
                                                         lmax=1000, npicard=51)),
}


def block_node_ids(mesh, ndof, seed):
    """Node numbering of Fill_ID.c (03_Euler_Equations/2D): dofs numbered node
    by node; inflow (x = 0) nodes have every dof prescribed, wall (y = 0) nodes
    their normal velocity (dof 2), a few random interior dofs are prescribed
    too so that mixed nodes occur."""
    rng = np.random.default_rng(seed)
    presc = np.zeros((mesh.nnodes, ndof), bool)
    presc[mesh.x == 0.0, :] = True
    presc[mesh.y == 0.0, 2 % ndof] = True
    presc |= rng.random((mesh.nnodes, ndof)) < 0.03
    node_id = np.full((mesh.nnodes, ndof), -1, np.int32)
    neq = 0
    for i in range(mesh.nnodes):
        for k in range(ndof):
            if not presc[i, k]:
                node_id[i, k] = neq
                neq += 1
    return node_id, neq


def run_ref_block(ndof, mesh, seed):
    name = "libfemref_euler_blk.so" if ndof == 4 else "libfemref_ns_blk.so"
    lib = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", name))
    f = lib.ref_block_run
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, ctypes.c_int, _ip, _ip, ctypes.c_int, _dp, _dp, _dp, _dp, _dp, _dp,
                  _dp, _dp, _dp, _dp]
    node_id, neq = block_node_ids(mesh, ndof, seed)
    m = 3 * ndof
    rng = np.random.default_rng(seed + 1)
    # diagonally weighted random element matrices keep the nodal blocks invertible
    A = rng.uniform(-1.0, 1.0, (mesh.nel, m, m)) + np.eye(m)[None] * 4.0
    P = rng.uniform(-1.0, 1.0, neq + 1)
    P[neq] = 0.0
    p = rng.uniform(-1.0, 1.0, neq + 1)
    p[neq] = 0.0
    F = rng.uniform(-1.0, 1.0, neq + 1)
    F[neq] = 0.0
    F0 = F.copy()
    d2 = ndof * ndof
    Q = np.zeros(neq + 1)
    Q2 = np.zeros(neq + 1)
    Q2no = np.zeros(neq + 1)
    BD = np.zeros(mesh.nnodes * d2)
    invBD = np.zeros(mesh.nnodes * d2)
    Z = np.zeros(neq + 1)
    f(mesh.nnodes, mesh.nel, np.ascontiguousarray(mesh.vert.reshape(-1)), node_id.reshape(-1), neq,
      np.ascontiguousarray(A.reshape(-1)), P, Q, Q2, Q2no, F, BD, invBD, p, Z)
    return dict(ndof=ndof, neq=neq, node_id=node_id, A=A.reshape(mesh.nel, m * m), P=P, Q=Q, Q2=Q2,
                Q2no=Q2no, F0=F0, F=F, BD=BD.reshape(mesh.nnodes, d2),
                invBD=invBD.reshape(mesh.nnodes, d2), p=p, Z=Z)


BLOCK_CASES = {"blk_euler_10x6": (4, 10, 6, 0.1, 11), "blk_ns_9x7": (3, 9, 7, 0.1, 12)}


def main_blocks():
    for name, (ndof, nx, ny, pert, seed) in BLOCK_CASES.items():
        mesh = structured_mesh(nx, ny, perturb=pert, seed=seed)
        out = run_ref_block(ndof, mesh, seed)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), x=mesh.x, y=mesh.y, vert=mesh.vert, **out)
        print(f"{name}: neq={out['neq']}")


# 2D Euler (REFLETIDO) cases: name -> (nx, ny, perturb, seed, alpha, CFL, stab_tol, nsteps, ncorr)
EULER_CASES = {
    "eul_refletido_16x4": (16, 4, 0.2, 3, 0.5, 5.0, 1e-6, 3, 2),
    "eul_refletido_12x6": (12, 6, 0.0, 4, 0.7, 2.0, 1e-3, 2, 3),
}


# Y^-1 of the YZBeta cases: 1 / the REFLETIDO inflow state (1 for its zero v)
YZ_INVY = np.array([1.0, 1.0 / 2.9, 1.0, 1.0 / 5.990715])


def main_euler():
    """Euler SUPG+CAU Build on a perturbed state (element matrices and
    residual) and a short predictor-multicorrector run, through the
    reference's sources (oracle/ref_euler_harness.c)."""
    from fem_codes_gb300.mesh import euler_cfl_dt, refletido_problem
    lib = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libfemref_euler.so"))
    lib.ref_euler_build.argtypes = [ctypes.c_int, _dp, _dp, _ip, ctypes.c_int, _ip, ctypes.c_int,
                                    ctypes.c_double, ctypes.c_double, ctypes.c_double, _dp, _dp, _dp, _dp]
    lib.ref_euler_predictor.argtypes = [ctypes.c_int, _dp, _dp, _ip, ctypes.c_int, _ip, ctypes.c_int,
                                        ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                                        ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_int, _dp, _dp,
                                        _ip]
    lib.ref_euler_predictor_csr.argtypes = lib.ref_euler_predictor.argtypes
    lib.ref_euler_build_scaled.argtypes = lib.ref_euler_build.argtypes
    lib.ref_euler_predictor_scaled.argtypes = lib.ref_euler_predictor.argtypes
    lib.ref_euler_build_slip.argtypes = [ctypes.c_int, _dp, _dp, _ip, _ip, ctypes.c_int, _ip, ctypes.c_int,
                                         ctypes.c_double, ctypes.c_double, ctypes.c_double, _dp, _dp, _dp, _dp,
                                         _dp, _dp]
    lib.ref_euler_set_shock.argtypes = [ctypes.c_int, _dp]
    lib.ref_euler_set_dd.argtypes = [ctypes.c_int]
    lib.ref_euler_build_dd.argtypes = [ctypes.c_int, _dp, _dp, _ip, ctypes.c_int, _ip, ctypes.c_int, ctypes.c_double,
                                       ctypes.c_double, ctypes.c_double, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp]
    lib.ref_euler_predictor_tint.restype = ctypes.c_int
    lib.ref_euler_predictor_tint.argtypes = [ctypes.c_int, ctypes.c_int, _dp, _dp, _ip, ctypes.c_int, _ip,
                                             ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                             ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                             ctypes.c_int, _dp, ctypes.c_int, _dp, _ip]
    lib.ref_euler_build2.argtypes = [ctypes.c_int, _dp, _dp, _ip, ctypes.c_int, _ip, ctypes.c_int, ctypes.c_double,
                                     ctypes.c_double, ctypes.c_double, _dp, _dp, _dp, _dp, _dp, _dp, _dp]
    lib.ref_euler_build_csr.restype = ctypes.c_int
    lib.ref_euler_build_csr.argtypes = [ctypes.c_int, _dp, _dp, _ip, ctypes.c_int, _ip, ctypes.c_int,
                                        ctypes.c_double, ctypes.c_double, ctypes.c_double, _dp, _dp, ctypes.c_int,
                                        _ip, _ip, _ip, _dp, _dp, _dp, _dp, _dp]
    for name, (nx, ny, pert, seed, alpha, cfl, stol, nsteps, ncorr) in EULER_CASES.items():
        mesh = structured_mesh(nx, ny, lx=4.0, ly=1.0, perturb=pert, seed=seed)
        pb = refletido_problem(mesh)
        neq = pb.neq
        rng = np.random.default_rng(seed)
        u = pb.u0 * (1.0 + 0.05 * rng.uniform(-1.0, 1.0, neq + 1))
        du = 0.1 * rng.uniform(-1.0, 1.0, neq + 1)
        u[neq] = du[neq] = 0.0
        dt = euler_cfl_dt(mesh, cfl)
        vert = np.ascontiguousarray(mesh.vert.reshape(-1), np.int32)
        nid = np.ascontiguousarray(pb.node_id.reshape(-1), np.int32)
        Ae = np.zeros(mesh.nel * 144)
        R = np.zeros(neq + 1)
        lib.ref_euler_build(mesh.nnodes, mesh.x, mesh.y, nid, mesh.nel, vert, neq, alpha, dt, stol, u, du,
                            Ae, R)
        kmax, lmax, tol = 30, 100, 1e-8
        up = pb.u0.copy()
        uhist = np.zeros(nsteps * (neq + 1))
        iters = np.zeros(nsteps * ncorr, np.int32)
        lib.ref_euler_predictor(mesh.nnodes, mesh.x, mesh.y, nid, mesh.nel, vert, neq, alpha, dt, stol,
                                kmax, lmax, tol, nsteps, ncorr, up, uhist, iters)
        # CSR storage with ILU(0): pattern, slot map, assembled values, R := M^-1 R,
        # one ILU(0) application, and the predictor run with ILU(0)-GMRES
        cap = 144 * mesh.nel
        IA = np.zeros(neq + 1, np.int32)
        JA = np.zeros(cap, np.int32)
        sbe = np.zeros(144 * mesh.nel, np.int32)
        AA = np.zeros(cap + 1)
        Rc = np.zeros(neq + 1)
        Rp = np.zeros(neq + 1)
        pz = rng.uniform(-1.0, 1.0, neq + 1)
        pz[neq] = 0.0
        zc = np.zeros(neq + 1)
        nnz = lib.ref_euler_build_csr(mesh.nnodes, mesh.x, mesh.y, nid, mesh.nel, vert, neq, alpha, dt, stol, u,
                                      du, cap, IA, JA, sbe, AA, Rc, Rp, pz, zc)
        assert nnz > 0
        upc = pb.u0.copy()
        uhc = np.zeros(nsteps * (neq + 1))
        itc = np.zeros(nsteps * ncorr, np.int32)
        lib.ref_euler_predictor_csr(mesh.nnodes, mesh.x, mesh.y, nid, mesh.nel, vert, neq, alpha, dt, stol,
                                    kmax, lmax, tol, nsteps, ncorr, upc, uhc, itc)
        amg_Fp = amg_fprec(IA, JA[:nnz], AA[:nnz], Rc[:neq], AMG_SYS_SPEC)
        # slip walls: the bottom wall's nodes whose v1 is free and v2 prescribed get
        # v1Type = -1 (Build_M_K_F_SUPG.c:1044-1056, rotation.c)
        slip = ((mesh.y == 0.0) & (pb.node_id[:, 1] >= 0) & (pb.node_id[:, 2] < 0)).astype(np.int32)
        Ae_s, R_s = np.zeros(mesh.nel * 144), np.zeros(neq + 1)
        cs, sn = np.zeros(mesh.nnodes), np.zeros(mesh.nnodes)
        lib.ref_euler_build_slip(mesh.nnodes, mesh.x, mesh.y, nid, slip, mesh.nel, vert, neq, alpha, dt, stol, u,
                                 du, Ae_s, R_s, cs, sn)
        # Scaling "BlockScaling": Block_scaling_EBE after the Build, and the predictor with it
        Ae_b, R_b = np.zeros(mesh.nel * 144), np.zeros(neq + 1)
        lib.ref_euler_build_scaled(mesh.nnodes, mesh.x, mesh.y, nid, mesh.nel, vert, neq, alpha, dt, stol, u, du,
                                   Ae_b, R_b)
        ups = pb.u0.copy()
        uhs = np.zeros(nsteps * (neq + 1))
        its_s = np.zeros(nsteps * ncorr, np.int32)
        lib.ref_euler_predictor_scaled(mesh.nnodes, mesh.x, mesh.y, nid, mesh.nel, vert, neq, alpha, dt, stol,
                                       kmax, lmax, tol, nsteps, ncorr, ups, uhs, its_s)
        # ShockCapture "YZBeta" (Delta_YZBeta.c) with Y^-1 from the inflow state: two consecutive
        # Builds from a zero delta_old (the second blends the first's delta) and the predictor
        lib.ref_euler_set_shock(1, YZ_INVY)
        Ae_y1, R_y1, Ae_y2, R_y2 = (np.zeros(mesh.nel * 144), np.zeros(neq + 1), np.zeros(mesh.nel * 144),
                                    np.zeros(neq + 1))
        dold_y = np.zeros(mesh.nel)
        lib.ref_euler_build2(mesh.nnodes, mesh.x, mesh.y, nid, mesh.nel, vert, neq, alpha, dt, stol, u, du,
                             Ae_y1, R_y1, Ae_y2, R_y2, dold_y)
        upy = pb.u0.copy()
        uhy = np.zeros(nsteps * (neq + 1))
        its_y = np.zeros(nsteps * ncorr, np.int32)
        lib.ref_euler_predictor(mesh.nnodes, mesh.x, mesh.y, nid, mesh.nel, vert, neq, alpha, dt, stol,
                                kmax, lmax, tol, nsteps, ncorr, upy, uhy, its_y)
        lib.ref_euler_set_shock(0, np.ones(4))
        # TimeIntegration Predictor1_BDF (3 time checks: 4 stages) and Predictor1_TRBDF2 (2 checks:
        # 4 stages) through the reference's own loops
        tint = {}
        for key, trbdf2, checks in (("bdf", 0, 3), ("tr", 1, 2)):
            cap = 8
            uht = np.zeros(cap * (neq + 1))
            itt = np.zeros(cap * ncorr, np.int32)
            st = lib.ref_euler_predictor_tint(trbdf2, mesh.nnodes, mesh.x, mesh.y, nid, mesh.nel, vert, neq, alpha,
                                              dt, stol, kmax, lmax, tol, checks, ncorr, pb.u0, cap, uht, itt)
            tint[key + "_uhist"] = uht[:st * (neq + 1)].reshape(st, neq + 1)
            tint[key + "_iters"] = itt[:st * ncorr].reshape(st, ncorr)
        # StabilizationForm "DD" (Build_M_K_F_DD_Transiente): two consecutive builds from seeded element
        # bubbles and a zero delta_old, with Delta_DD ("dd") and with Delta_YZBeta ("ddyz"), and the
        # Predictor_Old run with the DD build and Delta_DD
        dd = {}
        uB0 = rng.uniform(0.5, 1.5, 4 * mesh.nel)
        for key, yz in (("dd", 0), ("ddyz", 1)):
            lib.ref_euler_set_shock(yz, YZ_INVY if yz else np.ones(4))
            outs = [np.zeros(mesh.nel * 144), np.zeros(neq + 1), np.zeros(mesh.nel * 144), np.zeros(neq + 1),
                    np.zeros(4 * mesh.nel), np.zeros(mesh.nel)]
            lib.ref_euler_build_dd(mesh.nnodes, mesh.x, mesh.y, nid, mesh.nel, vert, neq, alpha, dt, stol, u, du,
                                   uB0, *outs)
            for k, v in zip(("Ae1", "R1", "Ae2", "R2", "uB", "dold"), outs):
                dd[f"{key}_{k}"] = v.reshape(mesh.nel, 144) if k.startswith("Ae") else v
        lib.ref_euler_set_shock(0, np.ones(4))
        dd["dd_uB0"] = uB0
        lib.ref_euler_set_dd(1)
        upd = pb.u0.copy()
        uhd = np.zeros(nsteps * (neq + 1))
        its_d = np.zeros(nsteps * ncorr, np.int32)
        lib.ref_euler_predictor(mesh.nnodes, mesh.x, mesh.y, nid, mesh.nel, vert, neq, alpha, dt, stol,
                                kmax, lmax, tol, nsteps, ncorr, upd, uhd, its_d)
        lib.ref_euler_set_dd(0)
        dd["dd_uhist"] = uhd.reshape(nsteps, neq + 1)
        dd["dd_iters"] = its_d.reshape(nsteps, ncorr)
        np.savez_compressed(
            os.path.join(HERE, f"{name}.npz"), x=mesh.x, y=mesh.y, vert=mesh.vert, node_id=pb.node_id,
            amg_spec=np.array(AMG_SYS_SPEC), amg_Fp=amg_Fp, **dd,
            bs_Ae=Ae_b.reshape(mesh.nel, 144), bs_R=R_b, bs_uhist=uhs.reshape(nsteps, neq + 1),
            bs_iters=its_s.reshape(nsteps, ncorr),
            yz_invY=YZ_INVY, yz_Ae1=Ae_y1.reshape(mesh.nel, 144), yz_R1=R_y1, yz_Ae2=Ae_y2.reshape(mesh.nel, 144),
            yz_R2=R_y2, yz_dold=dold_y, yz_uhist=uhy.reshape(nsteps, neq + 1), yz_iters=its_y.reshape(nsteps, ncorr),
            **tint,
            slip=slip, slip_cs=cs, slip_sn=sn, slip_Ae=Ae_s.reshape(mesh.nel, 144), slip_R=R_s,
            neq=neq, upresc=pb.upresc, u0=pb.u0, gamma=pb.gamma, alpha=alpha, dt=dt, stab_tol=stol,
            u=u, du=du, Ae=Ae.reshape(mesh.nel, 144), R=R, kmax=kmax, lmax=lmax, tol=tol,
            nsteps=nsteps, ncorr=ncorr, uhist=uhist.reshape(nsteps, neq + 1),
            iters=iters.reshape(nsteps, ncorr),
            csr_IA=IA, csr_JA=JA[:nnz], csr_sbe=sbe.reshape(mesh.nel, 144), csr_AA=AA[: nnz + 1], csr_R=Rc,
            csr_Rp=Rp, csr_p=pz, csr_z=zc, csr_uhist=uhc.reshape(nsteps, neq + 1),
            csr_iters=itc.reshape(nsteps, ncorr))
        print(f"{name}: neq={neq} nel={mesh.nel} dt={dt:.4g} iters={list(iters)} nnz={nnz} csr iters={list(itc)}")


# Navier-Stokes (CAVITY) cases: name -> (n, perturb, seed, Re, Newton iterations, forcing case)
NS_CASES = {
    "ns_cavity_10x10": (10, 0.0, 5, 100.0, 6, 2),
    "ns_cavity_12x12p": (12, 0.2, 6, 400.0, 5, 1),
}


def ns_lib():
    """A fresh copy of the reference NS library: Build_K_F_MS counts its calls
    in a file-scope variable, so every run needs its own instance."""
    import shutil
    import tempfile
    d = tempfile.mkdtemp()
    path = os.path.join(d, "libfemref_ns.so")
    shutil.copy(os.path.join(ROOT, "oracle", "_ref", "libfemref_ns.so"), path)
    L = ctypes.CDLL(path)
    L.ref_ns_builds.argtypes = [ctypes.c_int, _dp, _dp, _ip, ctypes.c_int, _ip, ctypes.c_int, ctypes.c_double,
                                ctypes.c_double, ctypes.c_int, _dp, _dp, _dp, _dp, _dp]
    L.ref_ns_newton.argtypes = [ctypes.c_int, _dp, _dp, _ip, ctypes.c_int, _ip, ctypes.c_int, ctypes.c_double,
                                ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                ctypes.c_double, ctypes.c_int, _dp, _dp, _dp, _ip]
    L.ref_ns_newton.restype = ctypes.c_int
    L.ref_ns_newton_csr.argtypes = L.ref_ns_newton.argtypes
    L.ref_ns_newton_csr.restype = ctypes.c_int
    L.ref_ns_builds_csr.argtypes = [ctypes.c_int, _dp, _dp, _ip, ctypes.c_int, _ip, ctypes.c_int, ctypes.c_double,
                                    ctypes.c_double, ctypes.c_int, _dp, ctypes.c_int, _ip, _ip, _dp, _dp, _dp, _dp,
                                    _dp]
    L.ref_ns_builds_csr.restype = ctypes.c_int
    L.CAVITY_v1presc.argtypes = [ctypes.c_double, ctypes.c_double]
    L.CAVITY_v1presc.restype = ctypes.c_double
    return L


def main_ns():
    """Three consecutive VMS builds on perturbed states (element matrices,
    residuals, stabilisation state) and a damped-Newton run, through the
    reference's sources (oracle/ref_ns_harness.c)."""
    from fem_codes_gb300.mesh import cavity_problem
    for name, (n, pert, seed, re, maxit, ecase) in NS_CASES.items():
        mesh = structured_mesh(n, n, perturb=pert, seed=seed)
        pb = cavity_problem(mesh, re)
        L = ns_lib()
        # the lid values exactly as the reference's plug-in computes them
        up = pb.upresc.copy()
        up[:, 0] = [L.CAVITY_v1presc(float(a), float(b)) for a, b in zip(mesh.x, mesh.y)]
        neq = pb.neq
        rng = np.random.default_rng(seed)
        us = np.zeros((3, neq + 1))
        for b in range(3):
            us[b, :neq] = 0.3 * rng.uniform(-1.0, 1.0, neq)
        vert = np.ascontiguousarray(mesh.vert.reshape(-1), np.int32)
        nid = np.ascontiguousarray(pb.node_id.reshape(-1), np.int32)
        Ae = np.zeros(3 * mesh.nel * 81)
        F = np.zeros(3 * (neq + 1))
        dold = np.zeros(mesh.nel)
        nold = np.zeros(mesh.nel)
        L.ref_ns_builds(mesh.nnodes, mesh.x, mesh.y, nid, mesh.nel, vert, neq, re, 1.0, 3, us.reshape(-1), Ae, F,
                        dold, nold)
        kmax, lmax, eta0, tolnl = 30, 50, 0.1, 1e-6
        L2 = ns_lib()
        uh = np.zeros(maxit * (neq + 1))
        nF = np.zeros(maxit)
        w = np.zeros(maxit)
        g = np.zeros(maxit, np.int32)
        nit = L2.ref_ns_newton(mesh.nnodes, mesh.x, mesh.y, nid, mesh.nel, vert, neq, re, 1.0, kmax, lmax, eta0,
                               ecase, tolnl, maxit, uh, nF, w, g)
        # CSR storage with ILU(0): pattern, three builds' assembled values,
        # F := M^-1 F, one ILU(0) application, and the damped-Newton run
        cap = 81 * mesh.nel
        cIA, cJA = np.zeros(neq + 1, np.int32), np.zeros(cap, np.int32)
        cAA, cF = np.zeros(3 * (cap + 1)), np.zeros(3 * (neq + 1))
        cFp, cz = np.zeros(neq + 1), np.zeros(neq + 1)
        cp = np.zeros(neq + 1)
        cp[:neq] = rng.uniform(-1.0, 1.0, neq)
        nnz = ns_lib().ref_ns_builds_csr(mesh.nnodes, mesh.x, mesh.y, nid, mesh.nel, vert, neq, re, 1.0, 3,
                                         us.reshape(-1), cap, cIA, cJA, cAA, cF, cFp, cp, cz)
        cAA = cAA.reshape(3, cap + 1)[:, : nnz + 1]
        cuh = np.zeros(maxit * (neq + 1))
        cnF, cw, cg = np.zeros(maxit), np.zeros(maxit), np.zeros(maxit, np.int32)
        cnit = ns_lib().ref_ns_newton_csr(mesh.nnodes, mesh.x, mesh.y, nid, mesh.nel, vert, neq, re, 1.0, kmax,
                                          lmax, eta0, ecase, tolnl, maxit, cuh, cnF, cw, cg)
        # AMG_precond_setup (DPA) on the last build's CSR system: F := M^-1 F
        amg_Fp = amg_fprec(cIA, cJA[:nnz], cAA[2][:nnz], cF.reshape(3, neq + 1)[2][:neq], AMG_SYS_SPEC)
        np.savez_compressed(
            os.path.join(HERE, f"{name}.npz"), x=mesh.x, y=mesh.y, vert=mesh.vert, node_id=pb.node_id, neq=neq,
            amg_spec=np.array(AMG_SYS_SPEC), amg_Fp=amg_Fp,
            upresc=up, f=pb.f, re=re, velmax=1.0, us=us, Ae=Ae.reshape(3, mesh.nel, 81), F=F.reshape(3, neq + 1),
            delta_old=dold, normres_old=nold, kmax=kmax, lmax=lmax, eta0=eta0, ecase=ecase, tolnl=tolnl,
            maxit=maxit, uhist=uh.reshape(maxit, neq + 1)[:nit], normF=nF[:nit], w=w[:nit], gmres=g[:nit],
            csr_IA=cIA, csr_JA=cJA[:nnz], csr_AA=cAA, csr_F=cF.reshape(3, neq + 1), csr_Fp=cFp, csr_p=cp,
            csr_z=cz, csr_uhist=cuh.reshape(maxit, neq + 1)[:cnit], csr_normF=cnF[:cnit], csr_w=cw[:cnit],
            csr_gmres=cg[:cnit])
        print(f"{name}: neq={neq} nel={mesh.nel} newton={nit} |F|={nF[:nit]} gmres={g[:nit]}; "
              f"CSR nnz={nnz} ILU(0) newton={cnit} |F|={cnF[:cnit]} gmres={cg[:cnit]}")


# name -> (nx, ny, perturb, node rule, transport kwargs, AMG deck string)
AMG_CASES = {
    "amg_skew20x16_hmatch": (20, 16, 0.2, "inflow", dict(problem="SKEW"), "AMG 2 2 -1 1.0 2"),
    "amg_skew20x16_count": (20, 16, 0.2, "inflow", dict(problem="SKEW"), "AMG 2 2 0.25 1.0 2"),
    "amg_conv28x20_rcm": (28, 20, 0.1, "all", dict(problem="CONVECTION", reord="SYMRCM"), "AMG 2 3 -1 0.9 1"),
    "amg_reaction24_beta0": (24, 24, 0.0, "all", dict(problem="REACTION"), "AMG 2 1 0 1.2 3"),
}


def amg_lib():
    """A fresh copy of libfemref_amg.so (the reference keeps its AMG state
    and the matching's pair counter in globals)."""
    import shutil
    import tempfile
    d = tempfile.mkdtemp()
    path = os.path.join(d, "libfemref_amg.so")
    shutil.copy(os.path.join(ROOT, "oracle", "_ref", "libfemref_amg.so"), path)
    L = ctypes.CDLL(path)
    L.ref_amg_setup.argtypes = [ctypes.c_int, _ip, _ip, _dp, ctypes.c_char_p, _dp, _ip]
    L.ref_amg_level.argtypes = [ctypes.c_int, _ip, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                ctypes.c_void_p]
    L.ref_amg_apply.argtypes = [_dp, _dp]
    L.ref_amg_gmres.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, _dp, _dp]
    L.ref_amg_gmres.restype = ctypes.c_int
    return L


# the AMG deck string of the Navier-Stokes and Euler CSR cases (DPA, 2
# coarsening sweeps per level, beta -1: the half-approximate matching)
AMG_SYS_SPEC = "AMG 2 2 -1 1.0 2"


def amg_fprec(IA, JA, AA, F, spec):
    """AMG_precond_setup's F := M^-1 F on an assembled CSR system (n rows)."""
    n = IA.size - 1
    L = amg_lib()
    Fp = np.concatenate([np.ascontiguousarray(F, np.float64), [0.0]])
    info = np.zeros(5, np.int32)
    L.ref_amg_setup(n, np.ascontiguousarray(IA, np.int32), np.ascontiguousarray(JA, np.int32),
                    np.ascontiguousarray(AA, np.float64), spec.encode(), Fp, info)
    return Fp[:n].copy()


def main_amg():
    """AMG_precond_setup / AMG_precond (DPA) and the AMG-preconditioned
    pgmres on steady-transport CSR matrices built by the reference
    (oracle/ref_amg_harness.c): every level's CSR and matching, M^-1 F, two
    V-cycle applications and the GMRES solution."""
    lib = load_ref()
    for name, (nx, ny, pert, rule, kw, spec) in AMG_CASES.items():
        mesh = structured_mesh(nx, ny, perturb=pert, seed=99)
        out = run_ref(lib, mesh, node_types(mesh, rule), scheme="CSR", precond="NOT", npicard=1, **kw)
        IA, JA = out["IA"], out["JA"]
        n, nnz = IA.size - 1, JA.size
        AA = np.ascontiguousarray(out["Afirst"][:nnz])
        F0 = np.ascontiguousarray(out["Ffirst"][:n])
        L = amg_lib()
        F = np.concatenate([F0, [0.0]])
        info = np.zeros(5, np.int32)
        L.ref_amg_setup(n, IA, JA, AA, spec.encode(), F, info)
        levels = {}
        for l in range(int(info[0])):
            nn = np.zeros(2, np.int32)
            L.ref_amg_level(l, nn, None, None, None, None)
            a, b, c = np.zeros(nn[0] + 1, np.int32), np.zeros(nn[1], np.int32), np.zeros(nn[1])
            rm = np.zeros(nn[0] + 1, np.int32) if l < info[0] - 1 else None
            L.ref_amg_level(l, nn, a.ctypes.data_as(ctypes.c_void_p), b.ctypes.data_as(ctypes.c_void_p),
                            c.ctypes.data_as(ctypes.c_void_p),
                            None if rm is None else rm.ctypes.data_as(ctypes.c_void_p))
            levels.update({f"IA{l}": a, f"JA{l}": b, f"AA{l}": c})
            if rm is not None:
                levels[f"rm{l}"] = rm
        rng = np.random.default_rng(5)
        qs = rng.uniform(-1.0, 1.0, (2, n))
        zs = np.zeros((2, n))
        for k in range(2):
            L.ref_amg_apply(np.ascontiguousarray(qs[k]), zs[k])
        B = F.copy()
        X = np.zeros(n + 1)
        kmax, lmax, tol = 30, 200, 1e-8
        it = L.ref_amg_gmres(kmax, lmax, tol, B, X)
        ntype = node_types(mesh, rule)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), spec=np.array(spec), IA=IA, JA=JA, AA=AA, F=F0,
                            x=mesh.x, y=mesh.y, vert=mesh.vert, node_type=ntype, beta=out["beta"],
                            fsrc=out["fsrc"], upresc=out["upresc"], problem=np.array(kw["problem"]),
                            reord=np.array(kw.get("reord", "NOT")),
                            nlev=int(info[0]), Fprec=F[:n], q=qs, z=zs, kmax=kmax, lmax=lmax, tol=tol,
                            X=X[:n], iters=it, **levels)
        sizes = [levels[f"IA{l}"].size - 1 for l in range(int(info[0]))]
        print(f"{name}: n={n} nnz={nnz} levels={sizes} gmres={it}")


def main_vtu():
    """Paraview_Output.c on the reference's own final Picard iterate of the
    skew16_csr_ilu0_rcm run: the VTU file's bytes and the inputs."""
    import tempfile
    lib = load_ref()
    lib.ref_transport_vtu.restype = ctypes.c_int
    lib.ref_transport_vtu.argtypes = [ctypes.c_int, _dp, _dp, _ip, ctypes.c_int, _ip, ctypes.c_int, ctypes.c_int, _dp]
    nx, ny, pert, rule, kw = CASES["skew16_csr_ilu0_rcm"]
    mesh = structured_mesh(nx, ny, perturb=pert, seed=1234)
    out = run_ref(lib, mesh, node_types(mesh, rule), **kw)
    u = np.ascontiguousarray(out["uhist"][-1])
    with tempfile.TemporaryDirectory() as d:
        os.makedirs(os.path.join(d, "run"))
        os.makedirs(os.path.join(d, "03_output"))
        cwd = os.getcwd()
        os.chdir(os.path.join(d, "run"))
        try:
            lib.ref_transport_vtu(mesh.nnodes, mesh.x, mesh.y, np.ascontiguousarray(out["node_id"], np.int32),
                                  mesh.nel, np.ascontiguousarray(mesh.vert.reshape(-1), np.int32),
                                  PROBLEMS["SKEW"], out["neq"], u)
        finally:
            os.chdir(cwd)
        files = os.listdir(os.path.join(d, "03_output"))
        assert len(files) == 1
        data = open(os.path.join(d, "03_output", files[0]), "rb").read()
    np.savez_compressed(os.path.join(HERE, "vtu_skew16_rcm.npz"), x=mesh.x, y=mesh.y, vert=mesh.vert,
                        node_type=node_types(mesh, rule), node_id=out["node_id"], neq=out["neq"], u=u,
                        vtu=np.frombuffer(data, dtype=np.uint8))
    print(f"vtu_skew16_rcm: {len(data)} bytes")


# Transient transport (02_Transport_Equation/2D): problem -> (harness code, domain side, origin)
TT_PROBLEMS = {"CONE": (0, 10.0, 0.0), "CONE2": (1, 10.0, -5.0), "CARTOLA": (2, 1.0, 0.0), "PUDIM": (3, 2.0, -1.0)}
TT_BASE = dict(reord="NOT", precond="NOT", stab="SUPG", shock="CAU", hshock="2sqrtArea", stopmc="ITERATION",
               steady="NOT", tint="Predictor1", alpha=0.5, dt=0.1, final=1.0, nonlin_tol=1e-3, max_corr=2, time_tol=1e-6,
               stab_tol=1e-6, kmax=30, lmax=20, tol=1e-8, maxsteps=12)
TT_CASES = {
    "tt_cone16_csr_ilu0_supg_rcm": dict(problem="CONE", n=16, scheme="CSR", reord="SYMRCM", precond="ILU0"),
    "tt_cartola16_csr_ilu0_supg": dict(problem="CARTOLA", n=16, scheme="CSR", precond="ILU0", hshock="Option1",
                                       stopmc="NORM", max_corr=4, dt=0.01, final=0.1),
    "tt_cone2_16_csr_ilu0_dd_caudd": dict(problem="CONE2", n=16, scheme="CSR", reord="SYMRCM", precond="ILU0",
                                          stab="DD", shock="CAUDD", hshock="Option1", dt=0.05, final=0.5),
    "tt_cone16_ebe_diag_dd_caudd": dict(problem="CONE", n=16, scheme="EBE", precond="Diag", stab="DD",
                                        shock="CAUDD", stopmc="NORM", max_corr=4),
    # YZBeta with Option2 amplifies rounding differences about x3-5 per step on this
    # unpreconditioned run: 8 steps keep the device run within 1e-8 of the reference's
    "tt_pudim16_ede_not_supg_yzbeta": dict(problem="PUDIM", n=16, scheme="EDE", shock="YZBeta", hshock="Option2",
                                           steady="YES", time_tol=1e-3, dt=0.05, maxsteps=8),
    "tt_cone2_12_csr_diag_dd_cau": dict(problem="CONE2", n=12, scheme="CSR", precond="Diag", stab="DD",
                                        shock="CAU", dt=0.05, final=0.5),
    "tt_cone16_csr_ilu0_supg_bdf": dict(problem="CONE", n=16, scheme="CSR", reord="SYMRCM", precond="ILU0",
                                        tint="Predictor1_BDF", maxsteps=8),
    "tt_cone2_16_csr_ilu0_dd_trbdf2": dict(problem="CONE2", n=16, scheme="CSR", precond="ILU0", stab="DD",
                                           shock="CAUDD", tint="Predictor1_TRBDF2", dt=0.05, maxsteps=6),
    "tt_cartola16_ebe_diag_supg_trbdf2": dict(problem="CARTOLA", n=16, scheme="EBE", precond="Diag",
                                              tint="Predictor1_TRBDF2", dt=0.01, maxsteps=6),
    "tt_cone16_csr_ilu0_dd_predictor2": dict(problem="CONE", n=16, scheme="CSR", reord="SYMRCM", precond="ILU0",
                                             stab="DD", shock="CAUDD", tint="Predictor2"),
    "tt_cone2_12_ebe_diag_dd_predictor2": dict(problem="CONE2", n=12, scheme="EBE", precond="Diag", stab="DD",
                                               shock="CAU", hshock="Option1", tint="Predictor2", dt=0.05,
                                               final=0.5, stopmc="NORM", max_corr=3),
    "tt_cone16_csr_ilu0_dd_predictor2_bdf": dict(problem="CONE", n=16, scheme="CSR", reord="SYMRCM",
                                                 precond="ILU0", stab="DD", shock="CAUDD", tint="Predictor2_BDF",
                                                 maxsteps=8),
    "tt_cone2_12_ebe_diag_dd_predictor2_trbdf2": dict(problem="CONE2", n=12, scheme="EBE", precond="Diag",
                                                      stab="DD", shock="CAU", tint="Predictor2_TRBDF2", dt=0.05,
                                                      maxsteps=6),
}


def transient_lib():
    lib = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libfemref_transient.so"))
    f = lib.ref_transient_run
    f.restype = ctypes.c_int
    s, d, i = ctypes.c_char_p, ctypes.c_double, ctypes.c_int
    f.argtypes = [i, _dp, _dp, _ip, i, _ip, i, s, s, s, s, s, s, s, s, s, d, d, d, d, i, d, d, i, i, d,
                  _ip, _ip, _dp, _dp, _dp, _dp, _ip, _ip, _ip, _ip, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp,
                  i, _dp, _dp, _ip, _ip]
    return lib


def transient_mesh(problem, n):
    _, side, origin = TT_PROBLEMS[problem]
    # PUDIM's initial data sits on the line x = 0, which only the unperturbed mesh holds
    m = structured_mesh(n, n, lx=side, ly=side, perturb=0.0 if problem == "PUDIM" else 0.2, seed=1234)
    m.x = m.x + origin
    m.y = m.y + origin
    bnd = (np.isclose(m.x, origin) | np.isclose(m.x, origin + side) | np.isclose(m.y, origin)
           | np.isclose(m.y, origin + side))
    return m, np.where(bnd, 0, 1).astype(np.int32)


def run_transient(lib, name, case):
    c = dict(TT_BASE)
    c.update(case)
    m, ntype = transient_mesh(c["problem"], c["n"])
    nn, ne = m.nnodes, m.nel
    neq = int((ntype == 1).sum())
    cap = 16 * (nn + ne) + 16
    info = np.zeros(5, np.int32)
    node_id = np.zeros(nn, np.int32)
    beta, fsrc, upresc = np.zeros(2 * ne), np.zeros(3 * ne), np.zeros(nn)
    u0 = np.zeros(neq + 1)
    IA, JA, sbe, order = (np.zeros(cap, np.int32) for _ in range(4))
    rng = np.random.default_rng(7)
    ub = rng.uniform(-0.5, 1.5, neq + 1)
    dub = rng.uniform(-1.0, 1.0, neq + 1)
    ub[neq] = dub[neq] = 0.0
    ubB = rng.uniform(-0.5, 1.5, ne)
    dubB = rng.uniform(-1.0, 1.0, ne)
    A1, A2 = np.zeros(cap), np.zeros(cap)
    R1, R2 = np.zeros(neq + 1), np.zeros(neq + 1)
    ms = c["maxsteps"]
    cap = 2 * ms + 2
    uh, th = np.zeros(cap * (neq + 1)), np.zeros(ms)
    nc, its = np.zeros(cap, np.int32), np.zeros(cap * 64, np.int32)
    e = lambda v: v.encode()
    stages = lib.ref_transient_run(
        nn, m.x, m.y, ntype, ne, np.ascontiguousarray(m.vert.reshape(-1), np.int32), TT_PROBLEMS[c["problem"]][0],
        e(c["scheme"]), e(c["reord"]), e(c["precond"]), e(c["stab"]), e(c["shock"]), e(c["hshock"]),
        e(c["stopmc"]), e(c["steady"]), e(c["tint"]), c["alpha"], c["dt"], c["final"], c["nonlin_tol"], c["max_corr"],
        c["time_tol"], c["stab_tol"], c["kmax"], c["lmax"], c["tol"], info, node_id, beta, fsrc, upresc, u0,
        IA, JA, sbe, order, ub, dub, ubB, dubB, A1, R1, A2, R2, ms, uh, th, nc, its)
    neq_r, nnz, nedge = int(info[0]), int(info[1]), int(info[2])
    assert neq_r == neq
    nA = {"CSR": nnz + 1, "EDE": 4 * (nedge + 1), "EBE": 9 * ne}[c["scheme"]]
    out = dict(x=m.x, y=m.y, vert=m.vert, node_type=ntype, neq=neq, nnz=nnz, nedge=nedge, node_id=node_id,
               beta=beta.reshape(ne, 2), fsrc=fsrc.reshape(ne, 3), upresc=upresc, u0=u0, ub=ub, dub=dub,
               ubB=ubB, dubB=dubB,
               A1=A1[:nA], R1=R1, A2=A2[:nA], R2=R2, stages=stages, tchecks=int(info[4]),
               uhist=uh.reshape(cap, neq + 1)[:stages], thist=th[:int(info[4])], ncorr=nc[:stages],
               iters=its.reshape(cap, 64)[:stages], meta=np.array(repr(c)))
    if c["scheme"] == "CSR":
        out.update(IA=IA[:neq + 1], JA=JA[:nnz], sbe=sbe[:9 * ne].reshape(ne, 9))
    elif c["scheme"] == "EDE":
        out.update(lm2=JA[:2 * nedge].reshape(nedge, 2), ebe=sbe[:3 * ne].reshape(ne, 3),
                   order=order[:3 * ne].reshape(ne, 3))
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    print(f"{name}: neq={neq} stages={stages} time checks={int(info[4])} ncorr={nc[:stages].tolist()} "
          f"iters={its.reshape(cap, 64)[:stages, 0].tolist()}")


def main_transient(names=()):
    lib = transient_lib()
    for name, case in TT_CASES.items():
        if not names or name in names:
            run_transient(lib, name, case)


def main(only=()):
    """Every fixture, or (names given on the command line) only those
    steady-transport cases ("euler": only the Euler cases)."""
    if only == ("euler",):
        main_euler()
        return
    if only == ("ns",):
        main_ns()
        return
    if only == ("vtu",):
        main_vtu()
        return
    if only == ("transient",):
        main_transient()
        return
    if only and all(n in TT_CASES for n in only):
        main_transient(only)
        return
    if not only:
        main_transient()
        main_vtu()
        main_amg()
        main_ns()
        main_euler()
        main_blocks()
    lib = load_ref()
    for name, (nx, ny, pert, rule, kw) in CASES.items():
        if only and name not in only:
            continue
        mesh = structured_mesh(nx, ny, perturb=pert, seed=1234)
        ntype = node_types(mesh, rule)
        out = run_ref(lib, mesh, ntype, **kw)
        meta = dict(kw)
        meta.setdefault("problem", "SKEW")
        np.savez_compressed(
            os.path.join(HERE, f"{name}.npz"),
            nx=nx, ny=ny, x=mesh.x, y=mesh.y, vert=mesh.vert, node_type=ntype,
            meta=np.array(repr(meta)), **out)
        print(f"{name}: neq={out['neq']} nnz={out['nnzero']} nedge={out['nedge']} "
              f"picard={out['npicard_run']} iters={list(out['iters'])}")


if __name__ == "__main__":
    main(tuple(sys.argv[1:]))
