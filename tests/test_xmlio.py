"""G+Smo XML input (gismo_gb300.xmlio), CPU only.

* Round trip: a problem written as XML and read back has bitwise the same patches and topology,
  and so the same gsDofMapper numbering, sparsity pattern and (to summation order) matrix
  (oracle).
* The reference's own XML parsers (oracle/ref/xml_dump.cpp, built from the G+Smo sources) read
  the same patches, knots, control points, interfaces and boundary sides as xmlio, on files
  written here and on sample files of the G+Smo source tree. Skipped where that tree is absent.
* Refinement and degree elevation follow gsKnotVector::uniformRefine / degreeElevate, and a
  problem read from a two-patch sample file converges at the optimal rate under refinement."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from gismo_gb300 import problems as P
from gismo_gb300 import xmlio

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
MK = os.path.join(ROOT, "oracle", "ref")
SAMPLES = ["planar/two_squares.xml", "planar/lshape2d_3patches_tens.xml", "planar/lshape_p2.xml",
           "planar/hexagon_3p.xml", "volumes/fichera.xml"]


def _cases():
    return [P.cube_grid(n=2, n_elem=3, p=2, seed=4, kappa_modes=0),
            P.displaced_single_patch(2, (7, 5), (3, 2), 3, 0.05, kappa_modes=0)]


def test_round_trip(tmp_path):
    from oracle import oracle as O
    for prob in _cases():
        f = str(tmp_path / "p.xml")
        xmlio.write_xml(prob, f)
        back = xmlio.with_fields(xmlio.problem_from_xml(f), prob)
        assert len(back.patches) == len(prob.patches)
        for a, b in zip(prob.patches, back.patches):
            assert tuple(a.gdegree) == tuple(b.gdegree) and tuple(a.degree) == tuple(b.degree)
            for k in range(prob.dim):
                assert np.array_equal(a.gknots[k], b.gknots[k]) and np.array_equal(a.knots[k], b.knots[k])
            assert np.array_equal(a.coefs, b.coefs)
        assert sorted(back.interfaces) == sorted(prob.interfaces)
        assert sorted(back.dirichlet) == sorted(prob.dirichlet)
        o1, o2 = O.OracleProblem(prob), O.OracleProblem(back)
        o1.assemble()
        o2.assemble()
        assert np.array_equal(o1.dofmap(), o2.dofmap())
        (p1, c1, v1), (p2, c2, v2) = o1.csr(), o2.csr()
        assert np.array_equal(p1, p2) and np.array_equal(c1, c2)
        # values up to the summation order of the oracle's OpenMP scatter
        assert np.abs(v1 - v2).max() <= 1e-13 * np.abs(v1).max()


def _reference_tree():
    if shutil.which("make") is None or shutil.which("g++") is None:
        return None
    ref = subprocess.run(["make", "-s", "-C", MK, "print-ref"], capture_output=True, text=True).stdout.strip()
    if not ref or not os.path.isdir(os.path.join(ref, "src", "gsIO")):
        return None
    r = subprocess.run(["make", "-s", "-C", MK, "xmldump"], capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    return ref


def _dump(path):
    exe = os.path.join(ROOT, "oracle", "_ref", "gsxml")
    out = subprocess.run([exe, path], capture_output=True, text=True, timeout=60, check=True).stdout.splitlines()
    patches, ifaces, bnd, ids = [], [], [], None
    i = 0
    while i < len(out):
        w = out[i].split()
        if w[0] == "patch":
            d = int(w[2])
            degs, knots = [], []
            for k in range(d):
                kv = out[i + 1 + k].split()
                degs.append(int(kv[1]))
                knots.append(np.array([float(v) for v in kv[3:]]))
            m = int(out[i + 1 + d].split()[1])
            coefs = np.array([[float(v) for v in out[i + 2 + d + r].split()] for r in range(m)])
            patches.append((int(w[1]), degs, knots, coefs))
            i += 2 + d + m
            continue
        if w[0] == "ids":
            ids = [int(v) for v in w[1:]]
        elif w[0] == "interface":
            v = [int(x) for x in w[1:]]
            dd = (len(v) - 4) // 2
            ifaces.append((v[0], v[1], v[2], v[3], tuple(v[4:4 + dd]), tuple(bool(x) for x in v[4 + dd:])))
        elif w[0] == "boundary":
            bnd.append((int(w[1]), int(w[2])))
        i += 1
    return patches, ids, ifaces, bnd


def test_reference_reader_agrees(tmp_path):
    ref = _reference_tree()
    if ref is None:
        pytest.skip("G+Smo source tree not available")
    files = []
    for k, prob in enumerate(_cases()):
        f = str(tmp_path / f"w{k}.xml")
        xmlio.write_xml(prob, f)
        files.append(f)
    files += [os.path.join(ref, "filedata", s) for s in SAMPLES if os.path.exists(os.path.join(ref, "filedata", s))]
    assert len(files) >= 4
    for f in files:
        ours = xmlio.read_xml(f)
        patches, ids, ifaces, bnd = _dump(f)
        if ids is None:  # single geometry: the first one
            ids = [patches[0][0]]
            bnd = [(0, s) for s in P.all_sides(ours["dim"])]
        assert ours["ids"] == ids, f
        byid = {p[0]: p for p in patches}
        for (degs, knots, coefs), i in zip(ours["patches"], ids):
            _, rdegs, rknots, rcoefs = byid[i]
            assert list(degs) == rdegs, f
            assert all(np.array_equal(a, b) for a, b in zip(knots, rknots)), f
            assert np.array_equal(coefs, rcoefs), f
        assert ours["interfaces"] == ifaces, f
        assert ours["boundary"] == bnd, f


def test_refine_and_elevate_knots():
    p, t = xmlio._elevate(2, np.array([0, 0, 0, 0.5, 1, 1, 1.0]), 1)
    assert p == 3 and np.array_equal(t, [0, 0, 0, 0, 0.5, 0.5, 1, 1, 1, 1])
    t = xmlio._refine(np.array([0, 0, 0.25, 1, 1.0]), 1)
    assert np.array_equal(t, [0, 0, 0.125, 0.25, 0.625, 1, 1])


def test_two_patch_sample_converges():
    """u = sin(pi x) sin(pi y) with Dirichlet data on the two unit squares of the G+Smo sample
    (written here with the same layout): L2 error at rate p + 1 under refinement."""
    from oracle import oracle as O
    import tempfile
    sq = [P.identity_patch(2, (1, 1), (1, 1)), P.identity_patch(2, (1, 1), (1, 1))]
    sq[1].coefs = sq[1].coefs - np.array([1.0, 0.0])
    two = P.Problem(2, sq, interfaces=[(1, 2, 0, 1)], dirichlet=[])
    with tempfile.TemporaryDirectory() as td:
        f = os.path.join(td, "two.xml")
        xmlio.write_xml(two, f)
        errs = []
        for r in (2, 3, 4):
            prob = xmlio.problem_from_xml(f, refine=r, elevate=1)
            assert len(prob.dirichlet) == 6 and prob.interfaces == [(1, 2, 0, 1)]
            o = O.OracleProblem(prob)
            o.assemble()
            x, _, _, _ = o.solve_cg(1e-12, 5000)
            errs.append(o.l2_error(x))
    rates = np.log2(np.array(errs[:-1]) / np.array(errs[1:]))
    assert np.all(rates >= 2.8), (errs, rates)


def test_rejections_and_uniform_knots(tmp_path):
    """NURBS patches and permuted / reversed interfaces are outside the path (ValueError); a
    KnotVector in mode="uniform" expands to the open uniform knots of its csize."""
    nurbs = tmp_path / "nurbs.xml"
    nurbs.write_text('<xml><Geometry type="TensorNurbs2" id="0"></Geometry></xml>')
    with pytest.raises(ValueError, match="not supported"):
        xmlio.read_xml(str(nurbs))
    two = [P.identity_patch(2, (1, 1), (1, 1)), P.identity_patch(2, (1, 1), (1, 1))]
    two[1].coefs = two[1].coefs - np.array([1.0, 0.0])
    f = str(tmp_path / "two.xml")
    xmlio.write_xml(P.Problem(2, two, interfaces=[(1, 2, 0, 1)]), f)
    text = open(f).read().replace("1 2 0 1 0 1 1 1", "1 2 0 1 0 1 1 0")  # reverse the side direction
    bad = tmp_path / "rev.xml"
    bad.write_text(text)
    with pytest.raises(ValueError, match="permuted or reversed"):
        xmlio.problem_from_xml(str(bad))
    uni = tmp_path / "uni.xml"
    uni.write_text('<xml><Geometry type="TensorBSpline2" id="0"><Basis type="TensorBSplineBasis2">'
                   '<Basis type="BSplineBasis" index="0"><KnotVector degree="2" mode="uniform" csize="5"/></Basis>'
                   '<Basis type="BSplineBasis" index="1"><KnotVector degree="1">0 0 1 1</KnotVector></Basis>'
                   '</Basis><coefs geoDim="2">' + " ".join("0 0" for _ in range(10)) + '</coefs></Geometry></xml>')
    d = xmlio.read_xml(str(uni))
    degs, knots, coefs = d["patches"][0]
    assert degs == [2, 1] and np.array_equal(knots[0], [0, 0, 0, 1 / 3, 2 / 3, 1, 1, 1]) and coefs.shape == (10, 2)
    assert d["boundary"] == [(0, s) for s in P.all_sides(2)]


def test_refine_and_elevate_match_reference():
    """xmlio's degree elevation and uniform refinement give bitwise the reference's knot vectors
    (gsKnotVector::degreeElevate / uniformRefine run by oracle/ref/knot_ops.cpp) on seeded knot
    vectors with repeated interior knots and uneven spans."""
    if _reference_tree() is None:
        pytest.skip("G+Smo source tree not available")
    r = subprocess.run(["make", "-s", "-C", MK, "knotops"], capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    exe = os.path.join(ROOT, "oracle", "_ref", "gsknot")
    rng = np.random.default_rng(5)
    for case in range(12):
        p = int(rng.integers(1, 4))
        interior = np.sort(rng.uniform(0.0, 2.0, size=int(rng.integers(0, 5))))
        reps = rng.integers(1, p + 1, size=len(interior))
        t = np.concatenate([[0.0] * (p + 1), np.repeat(interior, reps), [2.0] * (p + 1)])
        e, nref = int(rng.integers(0, 3)), int(rng.integers(0, 3))
        out = subprocess.run([exe, str(p), str(e), str(nref)] + [repr(float(v)) for v in t], capture_output=True,
                             text=True, timeout=60, check=True).stdout.split()
        q, s = xmlio._elevate(p, t, e)
        s = xmlio._refine(s, nref)
        assert q == int(out[0]), case
        assert np.array_equal(s, np.array([float(v) for v in out[1:]])), (case, s, out)
