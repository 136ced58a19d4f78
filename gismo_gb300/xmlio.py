"""G+Smo XML files (the gsFileData format) for the problem inputs: tensor B-spline patches and the
MultiPatch topology, read into :class:`gismo_gb300.problems.Problem` and written back.

Reading follows the reference's XML readers:
  * ``<Geometry type="TensorBSpline2|3" id=..>`` with a ``TensorBSplineBasis`` of one
    ``BSplineBasis`` per direction (``index`` attribute) holding a ``KnotVector`` (``degree``
    attribute, knots as text, or ``mode="uniform"`` with ``csize``) and ``<coefs geoDim=..>`` rows,
    first parametric direction fastest (gsXml<gsTensorBSpline>, src/gsNurbs/gsTensorBSpline.hpp:644;
    gsXml<gsKnotVector>, src/gsNurbs/gsKnotVector.hpp:30-100);
  * ``<MultiPatch parDim=..>`` with ``patches`` (``id_range`` first last, or ``id_index`` list),
    ``boundary`` (patch side pairs) and ``interfaces`` (patch side patch side, then d direction-map
    entries and d orientation flags per interface); patch ids become positions in the patches list;
    both lists are sorted and duplicates dropped (gsXml<gsMultiPatch>, src/gsIO/gsXmlUtils.hpp:968-1050;
    internal::getInterfaces / getBoundaries, src/gsIO/gsXml.cpp:221-313);
  * a file with geometries but no MultiPatch section is one patch with every side a boundary
    (gsMultiPatch::addAutoBoundaries).

The discretisation basis is the geometry basis after ``elevate`` degree elevations (every knot's
multiplicity and the degree raised together, gsKnotVector::degreeElevate,
src/gsNurbs/gsKnotVector.hpp:937-941) and ``refine`` uniform refinements (the midpoint of every
non-empty span inserted, gsKnotVector::uniformRefine / getUniformRefinementKnots,
src/gsNurbs/gsKnotVector.hpp:820-834, 1048-1063), the order of gsMultiBasis set-ups in the
reference's examples. NURBS (rational) patches, surfaces in 3D (geoDim != parDim) and interfaces
with a permuted or reversed side direction are outside this path and raise ValueError.
"""
from __future__ import annotations

import copy
import re
import xml.etree.ElementTree as ET
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from . import problems as P


def _numbers(text: Optional[str], kind=float) -> List:
    return [kind(t) for t in (text or "").split()]


def _knot_vector(node: ET.Element) -> Tuple[int, np.ndarray]:
    p = int(node.get("degree"))
    if node.get("mode") == "uniform":
        csize = node.get("csize")
        if csize is None:
            raise ValueError("uniform KnotVector without csize")
        n = int(csize)
        interior = n - p - 1
        return p, P.open_uniform_knots(interior + 1, p)
    fmt = (node.get("format") or "ascii").lower()
    if fmt != "ascii":
        raise ValueError(f"KnotVector format {fmt!r} is not supported")
    return p, np.array(_numbers(node.text), dtype=np.float64)


def _geometry(node: ET.Element) -> Tuple[int, List[int], List[np.ndarray], np.ndarray]:
    gtype = node.get("type", "")
    if gtype not in ("TensorBSpline2", "TensorBSpline3"):
        raise ValueError(f"geometry type {gtype!r} is not supported (tensor B-splines in 2D/3D only)")
    d = int(gtype[-1])
    basis = node.find("Basis")
    if basis is None or basis.get("type") != f"TensorBSplineBasis{d}":
        raise ValueError(f"{gtype} without a TensorBSplineBasis{d}")
    comps = basis.findall("Basis")
    if len(comps) != d:
        raise ValueError(f"TensorBSplineBasis{d} needs {d} component bases")
    comps = sorted(comps, key=lambda b: int(b.get("index", "0")))
    degs, knots = [], []
    for b in comps:
        if b.get("type") != "BSplineBasis":
            raise ValueError("component bases must be BSplineBasis")
        kv = b.find("KnotVector")
        if kv is None:
            raise ValueError("BSplineBasis without a KnotVector")
        p, t = _knot_vector(kv)
        degs.append(p)
        knots.append(t)
    cn = node.find("coefs")
    if cn is None:
        raise ValueError("geometry without coefs")
    gd = int(cn.get("geoDim", str(d)))
    if gd != d:
        raise ValueError(f"geoDim {gd} != parDim {d}: surfaces are not supported")
    c = np.array(_numbers(cn.text), dtype=np.float64)
    ncoef = int(np.prod([len(t) - p - 1 for t, p in zip(knots, degs)]))
    if c.size != ncoef * d:
        raise ValueError(f"coefs: {c.size} numbers for {ncoef} control points of dimension {d}")
    return d, degs, knots, c.reshape(ncoef, d)


def read_xml(path: str) -> Dict:
    """The tensor B-spline geometries and the first MultiPatch section of a G+Smo XML file:
    ``{"dim", "patches": [(degrees, knots, coefs)], "ids", "interfaces": [(p1, s1, p2, s2, dirmap,
    orientation)], "boundary": [(p, s)]}`` with patch ids translated to positions."""
    with open(path, "r", encoding="utf-8") as fh:
        text = fh.read()
    # the reference's parser accepts text before the XML declaration; the declaration carries
    # nothing this reader needs
    root = ET.fromstring(re.sub(r"<\?xml[^>]*\?>", "", text, count=1).strip())
    geos: Dict[int, Tuple] = {}
    order: List[int] = []
    for k, g in enumerate(root.findall("Geometry")):
        gid = int(g.get("id", str(-1 - k)))
        geos[gid] = _geometry(g)
        order.append(gid)
    if not geos:
        raise ValueError("no Geometry in the file")
    mp = root.find("MultiPatch")
    if mp is None:
        gid = order[0]
        d = geos[gid][0]
        return dict(dim=d, ids=[gid], patches=[geos[gid][1:]], interfaces=[],
                    boundary=[(0, s) for s in P.all_sides(d)])
    d = int(mp.get("parDim"))
    pn = mp.find("patches")
    vals = _numbers(pn.text, int)
    if pn.get("type") == "id_range":
        ids = list(range(vals[0], vals[1] + 1))
    elif pn.get("type") == "id_index":
        ids = vals
    else:
        raise ValueError(f"MultiPatch patches type {pn.get('type')!r} is not supported")
    pos = {i: k for k, i in enumerate(ids)}
    for i in ids:
        if i not in geos:
            raise ValueError(f"no Geometry with id {i}")
        if geos[i][0] != d:
            raise ValueError(f"patch {i} is not {d}-dimensional")
    boundary = set()
    for bn in mp.findall("boundary"):
        v = _numbers(bn.text, int)
        for a in range(0, len(v) - 1, 2):
            boundary.add((pos[v[a]], v[a + 1]))
    interfaces = {}
    for inode in mp.findall("interfaces"):
        v = _numbers(inode.text, int)
        step = 4 + 2 * d
        for a in range(0, len(v) - step + 1, step):
            p1, s1, p2, s2 = pos[v[a]], v[a + 1], pos[v[a + 2]], v[a + 3]
            dmap = tuple(v[a + 4:a + 4 + d])
            orient = [bool(o) for o in v[a + 4 + d:a + 4 + 2 * d]]
            # the side's own direction records whether both sides sit at the same parameter
            # (boundaryInterface constructors, src/gsCore/gsBoundary.h:665-716)
            nd = P.side_direction(s1)
            orient[nd] = P.side_parameter(s1) == P.side_parameter(s2)
            key = ((p1, s1), (p2, s2))
            interfaces.setdefault(key, (p1, s1, p2, s2, dmap, tuple(orient)))
    return dict(dim=d, ids=ids, patches=[geos[i][1:] for i in ids],
                interfaces=[interfaces[k] for k in sorted(interfaces)], boundary=sorted(boundary))


def _elevate(p: int, t: np.ndarray, e: int) -> Tuple[int, np.ndarray]:
    if e <= 0:
        return p, t
    u, m = np.unique(t, return_counts=True)
    return p + e, np.repeat(u, m + e)


def _refine(t: np.ndarray, r: int) -> np.ndarray:
    for _ in range(r):
        u = np.unique(t)
        mids = [u[i] + (u[i + 1] - u[i]) / 2.0 for i in range(len(u) - 1)]
        t = np.sort(np.concatenate([t, np.array(mids, dtype=np.float64)]), kind="stable")
    return t


def problem_from_xml(path: str, refine: int = 0, elevate: int = 0, neumann: Sequence[Tuple[int, int]] = (),
                     name: str = "") -> "P.Problem":
    """A Poisson problem on the file's multipatch: discretisation basis from the geometry basis
    (``elevate`` degree elevations, then ``refine`` uniform refinements), conforming interfaces
    glued, Dirichlet u on every boundary side except those listed in ``neumann``. Fields default
    to the Poisson case (kappa = 1, u = prod sin(pi x_i)); set them on the returned Problem."""
    data = read_xml(path)
    d = data["dim"]
    patches = []
    for degs, knots, coefs in data["patches"]:
        bdeg, bkn = [], []
        for p, t in zip(degs, knots):
            q, s = _elevate(p, t, elevate)
            bdeg.append(q)
            bkn.append(_refine(s, refine))
        patches.append(P.Patch(d, tuple(bdeg), bkn, tuple(degs), [np.array(t) for t in knots],
                               np.ascontiguousarray(coefs)))
    ifaces = []
    for p1, s1, p2, s2, dmap, orient in data["interfaces"]:
        nd = P.side_direction(s1)
        if any(dmap[i] != i for i in range(d)) or not all(orient[i] for i in range(d) if i != nd):
            raise ValueError(f"interface {p1}:{s1}-{p2}:{s2} is permuted or reversed (identity interfaces only)")
        ifaces.append((p1, s1, p2, s2))
    neu = [tuple(x) for x in neumann]
    dirichlet = [b for b in data["boundary"] if b not in neu]
    return P.Problem(d, patches, interfaces=ifaces, dirichlet=dirichlet, neumann=neu,
                     name=name or path.rsplit("/", 1)[-1].rsplit(".", 1)[0])


def _fmt(v: float) -> str:
    return repr(float(v))


def write_xml(prob: "P.Problem", path: str) -> None:
    """The problem's geometry as a G+Smo XML file: one TensorBSpline geometry per patch (its
    geometry basis and control points) and a MultiPatch section with the interfaces (identity
    direction map and orientation) and every side that is not an interface as boundary."""
    d = prob.dim
    lines = ['<?xml version="1.0" encoding="UTF-8"?>', "<xml>"]
    for k, pt in enumerate(prob.patches):
        lines.append(f'  <Geometry type="TensorBSpline{d}" id="{k}">')
        lines.append(f'    <Basis type="TensorBSplineBasis{d}">')
        for a in range(d):
            lines.append(f'      <Basis type="BSplineBasis" index="{a}">')
            lines.append(f'        <KnotVector degree="{int(pt.gdegree[a])}">'
                         + " ".join(_fmt(v) for v in pt.gknots[a]) + "</KnotVector>")
            lines.append("      </Basis>")
        lines.append("    </Basis>")
        lines.append(f'    <coefs geoDim="{d}">')
        for row in np.asarray(pt.coefs):
            lines.append("      " + " ".join(_fmt(v) for v in row))
        lines.append("    </coefs>")
        lines.append("  </Geometry>")
    n = len(prob.patches)
    lines.append(f'  <MultiPatch parDim="{d}" id="{n}">')
    lines.append(f'    <patches type="id_range">0 {n - 1}</patches>')
    if prob.interfaces:
        ident = " ".join(str(i) for i in range(d)) + " " + " ".join("1" for _ in range(d))
        lines.append("    <interfaces>" + "\n".join(f"{a} {b} {c} {e} {ident}" for a, b, c, e in prob.interfaces)
                     + "</interfaces>")
    iside = {(a, b) for a, b, _, _ in prob.interfaces} | {(c, e) for _, _, c, e in prob.interfaces}
    bnd = [(k, s) for k in range(n) for s in P.all_sides(d) if (k, s) not in iside]
    lines.append("    <boundary>" + "\n".join(f"{a} {b}" for a, b in bnd) + "</boundary>")
    lines.append("  </MultiPatch>")
    lines.append("</xml>")
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")


def with_fields(prob: "P.Problem", like: "P.Problem") -> "P.Problem":
    """A copy of ``prob`` with the coefficient, source and exact-solution parameters of ``like``."""
    out = copy.copy(prob)
    for f in ("kappa_fourier", "kappa_const", "kappa_alpha", "kappa_scale", "kappa_amp", "kappa_k", "kappa_phase",
              "ufreq", "quA", "quB"):
        setattr(out, f, copy.deepcopy(getattr(like, f)))
    return out
