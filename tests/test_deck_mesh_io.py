"""Parameter decks and mesh files (no GPU): femgpu_deck_read /
femgpu_mesh_read read the drivers' input files the way their Preprocess
does.  A transport deck and mesh are written in the drivers' format
("value<TAB>:label" lines with CRLF endings as the reference's decks have
them; the mesh file <title>_<nnodes>_<nel>.dat); the library's reading is
checked against the values written and, where the reference tree exists,
against the reference's own Preprocess run on the same files (parameters,
nodes with their equation numbers, elements).  Euler and Navier-Stokes decks
(their preconditioner strings may hold blanks) are read back too, and the
deck strings map to the library's options."""
import ctypes
import os

import numpy as np
import pytest

import fem_codes_gb300 as fg
from fem_codes_gb300.mesh import skew_problem, structured_mesh

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_LIB = os.path.join(ROOT, "oracle", "_ref", "libfemref.so")

TRANSPORT_DECK = [("TEST", "Experiments"), ("SKEWIO", "Problem title"), ("1e-8", "Solver tolerance"),
                  ("1e-4", "Non linear tolerance"), ("1000", "Solver max iterations"),
                  ("30", "Krylov basis vectors"), ("GMRES", "Solver"), ("ILU0", "Preconditioner"),
                  ("NOT", "Scaling"), ("SYMRCM", "Reordering"), ("CSR", "Matrix vector product scheme"),
                  ("SUPG", "Stabilization form"), ("CAU", "Shock capture"), ("2sqrtArea", "h shock"),
                  ("NO", "Output flow")]


def write_case(tmp, nx=12, ny=8):
    m = structured_mesh(nx, ny, perturb=0.2, seed=3)
    p = skew_problem(m)
    title = "SKEWIO"
    run = tmp / "run"
    mesh_dir = tmp / "02_mesh"
    run.mkdir()
    mesh_dir.mkdir()
    (tmp / "03_output").mkdir()
    lines = TRANSPORT_DECK + [(str(m.nnodes), "nnodes"), (str(m.nel), "nel")]
    deck = run / "params.dat"
    deck.write_bytes("".join(f"{v}\t:{lab}\r\n" for v, lab in lines).encode())
    with open(mesh_dir / f"{title}_{m.nnodes}_{m.nel}.dat", "w") as f:
        f.write(f"{m.nnodes}\n")
        for a, b, t in zip(m.x, m.y, p.node_type):
            f.write(f"{a:.17g}\t{b:.17g}\t{t}\n")
        f.write(f"{m.nel}\n")
        for v in m.vert:
            f.write(f"{v[0]}\t{v[1]}\t{v[2]}\t-1\n")
    return m, p, deck, mesh_dir


def test_transport_deck_and_mesh_read(tmp_path):
    m, p, deck, mesh_dir = write_case(tmp_path)
    d = fg.read_deck(str(deck), "transport")
    dd = d.as_dict()
    assert dd["Experiments"] == "TEST" and dd["ProblemTitle"] == "SKEWIO" and dd["Preconditioner"] == "ILU0"
    assert dd["SolverTolerance"] == 1e-8 and dd["NonLinearTolerance"] == 1e-4
    assert dd["SolverMaxIter"] == 1000 and dd["KrylovBasisVectorsQuantity"] == 30
    assert dd["nnodes"] == m.nnodes and dd["nel"] == m.nel and dd["OutputFlow"] == "NO"
    path = fg.deck_mesh_file(d, str(mesh_dir))
    assert os.path.basename(path) == f"SKEWIO_{m.nnodes}_{m.nel}.dat"
    mesh = fg.read_mesh(path, "transport")
    assert np.array_equal(mesh["x"], m.x) and np.array_equal(mesh["y"], m.y)
    assert np.array_equal(mesh["node_type"], p.node_type) and np.array_equal(mesh["vert"], m.vert)
    o = fg.deck_opts(d)
    assert (o.scheme, o.reorder, o.precond, o.kmax, o.lmax, o.tol) == (2, 1, 1, 30, 1000, 1e-8)


@pytest.mark.skipif(not os.path.exists(REF_LIB), reason="the reference library is not built here")
def test_transport_reading_matches_reference_preprocess(tmp_path):
    m, p, deck, mesh_dir = write_case(tmp_path)
    L = ctypes.CDLL(REF_LIB)
    f = L.ref_transport_preprocess
    f.restype = ctypes.c_int
    nn, ne = m.nnodes, m.nel
    iv = np.zeros(6, np.int32)
    dv = np.zeros(2)
    sv = ctypes.create_string_buffer(64 * 11)
    x, y = np.zeros(nn), np.zeros(nn)
    t, ident = np.zeros(nn, np.int32), np.zeros(nn, np.int32)
    vert, et = np.zeros(3 * ne, np.int32), np.zeros(ne, np.int32)
    cwd = os.getcwd()
    os.chdir(tmp_path / "run")
    try:
        rc = f(str(deck).encode(), iv.ctypes.data_as(ctypes.c_void_p), dv.ctypes.data_as(ctypes.c_void_p), sv,
               x.ctypes.data_as(ctypes.c_void_p), y.ctypes.data_as(ctypes.c_void_p), t.ctypes.data_as(ctypes.c_void_p),
               ident.ctypes.data_as(ctypes.c_void_p), vert.ctypes.data_as(ctypes.c_void_p),
               et.ctypes.data_as(ctypes.c_void_p), nn, ne)
    finally:
        os.chdir(cwd)
    assert rc == 0
    d = fg.read_deck(str(deck), "transport").as_dict()
    strings = [sv.raw[64 * i:64 * (i + 1)].split(b"\0")[0].decode() for i in range(11)]
    assert strings == [d[k] for k in ("Experiments", "ProblemTitle", "Solver", "Preconditioner", "Scaling",
                                      "reordering", "MatrixVectorProductScheme", "StabilizationForm",
                                      "ShockCapture", "h_Shock", "OutputFlow")]
    assert [iv[0], iv[1], iv[3], iv[4]] == [d["nnodes"], d["nel"], d["SolverMaxIter"], d["KrylovBasisVectorsQuantity"]]
    assert list(dv) == [d["SolverTolerance"], d["NonLinearTolerance"]]
    mesh = fg.read_mesh(fg.deck_mesh_file(fg.read_deck(str(deck), "transport"), str(mesh_dir)), "transport")
    assert np.array_equal(mesh["x"], x) and np.array_equal(mesh["y"], y)
    assert np.array_equal(mesh["node_type"], t)
    assert np.array_equal(mesh["vert"].reshape(-1), vert) and np.array_equal(mesh["elem_type"], et)
    # the equation numbers of Preprocess.c:73-81, permuted by the reordering:
    # one per node of type >= 1, none elsewhere
    free = mesh["node_type"] >= 1
    assert iv[2] == free.sum() and np.all(ident[~free] == -1)
    assert np.array_equal(np.sort(ident[free]), np.arange(iv[2]))


def test_euler_and_ns_decks(tmp_path):
    eul = [("NCONG", "e"), ("REFLETIDO", "t"), ("1e-8", "tol"), ("1e-3", "nl"), ("1e-5", "ti"), ("1e-6", "stab"),
           ("100", "maxit"), ("50", "krylov"), ("GMRES", "solver")]
    text = "".join(f"{v}\t:{lab}\r\n" for v, lab in eul)
    text += "AMG 2 3 -1 1.0 2\t:Preconditioner\r\n"
    rest = [("NOT", "scaling"), ("NOT", "reord"), ("PREDICTOR1", "ti"), ("NOT", "steady"), ("0.5", "alpha"),
            ("5e-3", "dt"), ("1.0", "final"), ("NO", "dimless"), ("1.0", "mach"), ("2", "ncorr"),
            ("ITERATION", "stop"), ("CSR", "scheme"), ("SUPG", "stab"), ("CAU", "shock"), ("1", "y0"), ("1", "y1"),
            ("1", "y2"), ("1", "y3"), ("100", "nnodes"), ("162", "nel")]
    text += "".join(f"{v}\t:{lab}\r\n" for v, lab in rest)
    path = tmp_path / "eul.dat"
    path.write_bytes(text.encode())
    d = fg.read_deck(str(path), "euler")
    dd = d.as_dict()
    assert dd["Preconditioner"].startswith("AMG 2 3 -1 1.0 2") and dd["StopMulticorrection"] == "ITERATION"
    assert dd["DeltaT"] == 5e-3 and dd["NonLinearMaxIter"] == 2 and dd["nel"] == 162
    o = fg.deck_opts(d)
    assert (o.scheme, o.precond, o.kmax, o.lmax, o.ncorr, o.scaling) == (2, 5, 50, 100, 2, 0)
    assert (o.shock, list(o.invY)) == (0, [1.0, 1.0, 1.0, 1.0])
    # setStabilizationForm.c:27: ShockCapture YZBeta takes the deck's Y^-1
    t = text.replace("CAU\t:shock", "YZBeta\t:shock").replace("1\t:y1", "0.5\t:y1")
    path.write_bytes(t.encode())
    oy = fg.deck_opts(fg.read_deck(str(path), "euler"))
    assert (oy.shock, list(oy.invY)) == (1, [1.0, 0.5, 1.0, 1.0])
    # setStabilizationForm.c:9-21: the SUPG time loops
    for ti, method in (("PREDICTOR1_BDF", 1), ("Predictor1_TRBDF2", 2), ("Predictor2", None)):
        path.write_bytes(text.replace("PREDICTOR1\t:ti", f"{ti}\t:ti").encode())
        dt_ = fg.read_deck(str(path), "euler")
        if method is None:
            with pytest.raises(fg.FemGpuError):
                fg.deck_opts(dt_)
        else:
            assert fg.deck_opts(dt_).method == method
    # setScaling.c:6-27: BlockScaling with EBE storage, rejected with CSR
    for scheme, pre, ok in (("EBE", "BlockDiag", True), ("CSR", "ILU0", False)):
        t = text.replace("NOT\t:scaling", "BlockScaling\t:scaling").replace("CSR\t:scheme", f"{scheme}\t:scheme")
        t = t.replace("AMG 2 3 -1 1.0 2\t:Preconditioner", f"{pre}\t:Preconditioner")
        path.write_bytes(t.encode())
        db = fg.read_deck(str(path), "euler")
        assert db.as_dict()["Scaling"] == "BlockScaling"
        if ok:
            assert fg.deck_opts(db).scaling == 1
        else:
            with pytest.raises(fg.FemGpuError):
                fg.deck_opts(db)
    ns = [("E", "e"), ("CAVITY", "t"), ("1000", "re"), ("1", "vmax"), ("0.1", "tol"), ("2", "case"),
          ("1e-8", "nl"), ("50", "maxit"), ("30", "krylov"), ("GMRES", "solver")]
    text = "".join(f"{v}\t:{lab}\r\n" for v, lab in ns) + "ILU0\t:Preconditioner\r\n"
    text += "".join(f"{v}\t:{lab}\r\n" for v, lab in [("NOT", "r"), ("CSR", "s"), ("MS", "f"), ("121", "n"),
                                                        ("200", "e")])
    path = tmp_path / "ns.dat"
    path.write_bytes(text.encode())
    dn = fg.read_deck(str(path), "ns")
    o = fg.deck_opts(dn)
    assert (o.re, o.eta_case, o.scheme, o.precond, o.lmax) == (1000.0, 2, 2, 1, 50)


def test_bad_files_rejected(tmp_path):
    p = tmp_path / "bad.dat"
    p.write_text("3\n0 0 1\n1 0\n")
    with pytest.raises(fg.FemGpuError):
        fg.read_mesh(str(p), "transport")
    with pytest.raises(fg.FemGpuError):
        fg.read_deck(str(tmp_path / "missing.dat"), "transport")


TRANSIENT_REF_LIB = os.path.join(ROOT, "oracle", "_ref", "libfemref_transient.so")
TRANSIENT_DECK = [("CONE", "Problem title"), ("1e-8", "Solver tolerance"), ("1e-3", "Non linear tolerance"),
                  ("1e-4", "Time integration tolerance"), ("1e-6", "Stabilization tolerance"),
                  ("3", "Non linear max iterations"), ("200", "Linear max iterations"),
                  ("YES", "Stop at steady state"), ("25", "Krylov basis vectors"), ("GMRES", "Solver"),
                  ("ILU1", "Preconditioner"), ("NOT", "Scaling"), ("SYMRCM", "Reordering"),
                  ("CSR", "Matrix vector product scheme"), ("DD", "Stabilization form"),
                  ("CAUDD", "Shock capture"), ("Option1", "h shock"), ("Predictor2_TRBDF2", "Time integration"),
                  ("0.5", "Alpha"), ("0.05", "Delta t"), ("NORM", "Stop multicorrection"), ("1.5", "Final time")]


def write_transient_case(tmp, nx=10, ny=10, deck=TRANSIENT_DECK):
    """A transient transport deck and its mesh file where the driver's
    Preprocess looks for it: ../../../../INPUT_DATA from the run folder."""
    m = structured_mesh(nx, ny, perturb=0.2, seed=5)
    bnd = (m.x == 0.0) | (m.x == 1.0) | (m.y == 0.0) | (m.y == 1.0)
    ntype = np.where(bnd, 0, 1).astype(np.int32)
    run = tmp / "a" / "b" / "c" / "run"
    mesh_dir = tmp / "INPUT_DATA"
    run.mkdir(parents=True)
    mesh_dir.mkdir()
    lines = deck + [(str(m.nnodes), "nnodes"), (str(m.nel), "nel")]
    path = run / "params.dat"
    path.write_bytes("".join(f"{v}\t:{lab}\r\n" for v, lab in lines).encode())
    with open(mesh_dir / f"CONE_{m.nnodes}_{m.nel}.dat", "w") as f:
        f.write(f"{m.nnodes}\n")
        for a, b, t in zip(m.x, m.y, ntype):
            f.write(f"{a:.17g}\t{b:.17g}\t{t}\n")
        f.write(f"{m.nel}\n")
        for v in m.vert:
            f.write(f"{v[0]}\t{v[1]}\t{v[2]}\n")
    return m, ntype, path, mesh_dir


def test_transient_deck_mesh_and_options(tmp_path):
    """The transient driver's deck (02_Transport_Equation/2D Preprocess.c:
    42-66) and its mesh file without element types (Preprocess.c:94-97), and
    the deck strings as transport + transient options."""
    m, ntype, deck, mesh_dir = write_transient_case(tmp_path)
    d = fg.read_deck(str(deck), "transient")
    dd = d.as_dict()
    assert dd["ProblemTitle"] == "CONE" and dd["TimeIntegration"] == "Predictor2_TRBDF2"
    assert (dd["SolverTolerance"], dd["NonLinearTolerance"], dd["TimeIntegrationTolerance"],
            dd["StabilizationTolerance"], dd["Alpha"], dd["DeltaT"], dd["FinalTime"]) == \
        (1e-8, 1e-3, 1e-4, 1e-6, 0.5, 0.05, 1.5)
    assert (dd["NonLinearMaxIter"], dd["LinearMaxIter"], dd["KrylovBasisVectorsQuantity"]) == (3, 200, 25)
    assert (dd["StopAtSteadyState"], dd["StopMulticorrection"], dd["h_Shock"]) == ("YES", "NORM", "Option1")
    mesh = fg.read_mesh(fg.deck_mesh_file(d, str(mesh_dir)), "transient")
    assert np.array_equal(mesh["x"], m.x) and np.array_equal(mesh["y"], m.y)
    assert np.array_equal(mesh["node_type"], ntype) and np.array_equal(mesh["vert"], m.vert)
    assert not mesh["elem_type"].any()
    o, tr = fg.deck_opts(d)
    assert (o.scheme, o.reorder, o.precond, o.ilu_level, o.shock, o.kmax, o.lmax, o.tol) == \
        (2, 1, 1, 1, 2, 25, 200, 1e-8)
    assert (tr.stab, tr.method, tr.stop_norm, tr.steady_stop, tr.max_corr) == (1, 5, 1, 1, 3)
    assert (tr.alpha, tr.dt, tr.final_time, tr.nonlin_tol, tr.time_tol) == (0.5, 0.05, 1.5, 1e-3, 1e-4)
    # setStabilizationForm.c / setPreconditioner.c reject these combinations
    for key, val in (("Stabilization form", "SUPG"), ("Matrix vector product scheme", "EBE"),
                     ("Time integration", "Predictor3"), ("Stop multicorrection", "SOMETIMES")):
        bad = [(val if lab == key else v, lab) for v, lab in TRANSIENT_DECK]
        sub = tmp_path / key.replace(" ", "_")
        sub.mkdir()
        _, _, p, _ = write_transient_case(sub, deck=bad)
        with pytest.raises(fg.FemGpuError):
            fg.deck_opts(fg.read_deck(str(p), "transient"))


@pytest.mark.skipif(not os.path.exists(TRANSIENT_REF_LIB), reason="the reference library is not built here")
def test_transient_reading_matches_reference_preprocess(tmp_path):
    m, ntype, deck, mesh_dir = write_transient_case(tmp_path)
    L = ctypes.CDLL(TRANSIENT_REF_LIB)
    f = L.ref_transient_preprocess
    f.restype = ctypes.c_int
    nn, ne = m.nnodes, m.nel
    iv, dv = np.zeros(7, np.int32), np.zeros(7)
    sv = ctypes.create_string_buffer(64 * 13)
    x, y = np.zeros(nn), np.zeros(nn)
    t, ident = np.zeros(nn, np.int32), np.zeros(nn, np.int32)
    vert, et = np.zeros(3 * ne, np.int32), np.full(ne, 7, np.int32)
    vp = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    cwd = os.getcwd()
    os.chdir(deck.parent)
    try:
        rc = f(str(deck).encode(), vp(iv), vp(dv), sv, vp(x), vp(y), vp(t), vp(ident), vp(vert), vp(et), nn, ne)
    finally:
        os.chdir(cwd)
    assert rc == 0
    d = fg.read_deck(str(deck), "transient").as_dict()
    strings = [sv.raw[64 * i:64 * (i + 1)].split(b"\0")[0].decode() for i in range(12)]
    assert strings == [d[k] for k in ("ProblemTitle", "StopAtSteadyState", "Solver", "Preconditioner", "Scaling",
                                      "reordering", "MatrixVectorProductScheme", "StabilizationForm",
                                      "ShockCapture", "h_Shock", "TimeIntegration", "StopMulticorrection")]
    assert list(iv[[0, 1, 3, 4, 5]]) == [d["nnodes"], d["nel"], d["NonLinearMaxIter"], d["LinearMaxIter"],
                                         d["KrylovBasisVectorsQuantity"]]
    assert list(dv) == [d[k] for k in ("SolverTolerance", "NonLinearTolerance", "TimeIntegrationTolerance",
                                       "StabilizationTolerance", "Alpha", "DeltaT", "FinalTime")]
    mesh = fg.read_mesh(fg.deck_mesh_file(fg.read_deck(str(deck), "transient"), str(mesh_dir)), "transient")
    assert np.array_equal(mesh["x"], x) and np.array_equal(mesh["y"], y)
    assert np.array_equal(mesh["node_type"], t)
    assert np.array_equal(mesh["vert"].reshape(-1), vert) and np.array_equal(mesh["elem_type"], et)
    free = mesh["node_type"] >= 1
    assert iv[2] == free.sum() and np.all(ident[~free] == -1)
    assert np.array_equal(np.sort(ident[free]), np.arange(iv[2]))
