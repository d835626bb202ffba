"""Generate golden fixtures by running the reference's own Python setup modules.

Runs (in this container only; the output is committed):
  pyprop/bspline/gausslegendrequadrature.py   GaussQuadratureRule (nodes, weights)
  pyprop/bspline/breakpointsequences.py       Linear / Exponential / ExponentialLinear sequences
  pyprop/bspline/BSpline.py                   BSPLINE.CreateContinuitySequence, CreateKnotSequence,
                                              SetupQuadratureRule, SetupGlobalGridAndWeights,
                                              NumberOfBSplines
The modules are Python 2; the few Python-2-only statements they contain
(`raise E, "msg"`, `execfile`, `xrange`) are adapted textually before exec,
and the compiled base class core.BSpline is replaced by a plain holder of the
arrays those methods fill (plus ScaleAndTranslate, core/transform/bspline/bspline.h:173-176).
`frange` (matplotlib.mlab, imported by the reference through pylab) is
supplied with matplotlib's published semantics (closed interval, npts =
round((xfin - xini)/delta) + 1).

Writes tests/golden/setup_golden.npz.

It also runs the reference's storage and pair generators (pure Python):
  pyprop/tensorpotential/GeometryInfo.py        GeometryInfoCommonBandedNonHermitian.GetBasisPairs
  pyprop/tensorpotential/basis/ReducedSphericalHarmonic.py
                                                GeometryInfoReducedSphHarmSelectionRule.GetBasisPairs
with a stand-in for the compiled ReducedSphericalTools exposing GetSize() = LMax - |M|
(core/transform/reducedspherical/reducedsphericaltools.h:53), and writes
tests/golden/geometry_golden.npz; and the velocity-gauge pulse LaserFunctionVelocity of the
helium_stabilization_sae example -> tests/golden/laser_golden.npz.

Usage: python tests/golden/make_golden.py [REFERENCE_TREE]
The reference tree (a checkout of pyprop) is the first argument, else the environment variable
PYPROP_REFERENCE.
"""
from __future__ import annotations

import os
import re
import sys
import types

import numpy as np

def _reference_tree():
    path = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PYPROP_REFERENCE", "")
    if not path or not os.path.isdir(os.path.join(path, "pyprop")):
        sys.exit("usage: make_golden.py REFERENCE_TREE (or set PYPROP_REFERENCE): a pyprop checkout")
    return path


REF = _reference_tree() if __name__ == "__main__" else None
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "setup_golden.npz")


def _py2_to_py3(src):
    src = re.sub(r"raise\s+(\w+)\s*,\s*(.+)", r"raise \1(\2)", src)
    src = src.replace("(core.BSpline)", "(_RefCoreBSpline)")
    src = re.sub(r"^(\s*)print\s+(\".*)$", r"\1print(\2)", src, flags=re.M)
    return src


def _frange(xini, xfin=None, delta=None, **kw):
    endpoint = kw.get("closed", 1) != 0
    if xfin is None:
        xfin = xini + 0.0
        xini = 0.0
    if delta is None:
        delta = 1.0
    npts = int(np.round((xfin - xini) / delta)) + endpoint
    return np.arange(npts) * delta + xini


def load_modules():
    ns = {"__name__": "pyprop_ref", "xrange": range, "frange": _frange}
    exec("from numpy import *", ns)
    ns["frange"] = _frange

    def execfile(path, g=None, l=None):
        with open(path) as f:
            code = _py2_to_py3(f.read())
        exec(compile(code, path, "exec"), ns)

    ns["execfile"] = execfile
    ns["__path__"] = [os.path.join(REF, "pyprop")]

    class _CoreBSpline:
        """Holder of the arrays BSPLINE's Python methods fill."""

        def __init__(self):
            self._a = {}

        def _resize(self, name, n, dtype=float):
            self._a[name] = np.zeros(n, dtype=dtype)

        def _get(self, name):
            return self._a[name]

        ResizeBreakpointSequence = lambda self, n: self._resize("bp", n)
        GetBreakpointSequence = lambda self: self._get("bp")
        ResizeContinuitySequence = lambda self, n: self._resize("cont", n, int)
        GetContinuitySequence = lambda self: self._get("cont")
        ResizeKnotSequence = lambda self, n: self._resize("knots", n)
        GetKnotSequence = lambda self: self._get("knots")
        ResizeTopKnotMap = lambda self, n: self._resize("topknot", n, int)
        GetTopKnotMap = lambda self: self._get("topknot")
        ResizeWeights = lambda self, n: self._resize("weights", n)
        GetWeights = lambda self: self._get("weights")
        ResizeNodes = lambda self, n: self._resize("nodes", n)
        GetNodes = lambda self: self._get("nodes")
        ResizeQuadratureGridGlobal = lambda self, n: self._resize("grid", n)
        GetQuadratureGridGlobal = lambda self: self._get("grid")
        ResizeQuadratureWeightsGlobal = lambda self, n: self._resize("gw", n)
        GetQuadratureWeightsGlobal = lambda self: self._get("gw")
        ResizeKnotGridIndexMap = lambda self, n: self._resize("kgmap", n, int)
        GetKnotGridIndexMap = lambda self: self._get("kgmap")

        def ScaleAndTranslate(self, x, a, b):
            return (x - 1.0) * (b - a) / 2.0 + b

    ns["_RefCoreBSpline"] = _CoreBSpline
    execfile(os.path.join(REF, "pyprop", "bspline", "BSpline.py"))
    return ns


class _Conf:
    def __init__(self, **kw):
        self.__dict__.update(kw)

    def Get(self, k):
        return self.__dict__[k]


def main():
    ns = load_modules()
    out = {}
    for order in (2, 3, 5, 7, 9, 10, 11, 16):
        q = ns["GaussQuadratureRule"](ruleOrder=order)
        out["gl_nodes_%d" % order] = np.asarray(q.Nodes, dtype=float).real
        out["gl_weights_%d" % order] = np.asarray(q.Weights, dtype=float).real
    out["bp_linear"] = np.array(ns["LinearBreakpointSequence"](0.0, 50.0, 103))
    out["bp_exponential"] = np.array(ns["ExponentialBreakpointSequence"](0.0, 100.0, 60, 3.0))
    out["bp_explinear"] = np.array(ns["ExponentialLinearBreakpointSequence"](0.0, 20.0, 400.0, 60, 2.0))
    cases = {
        "small": dict(order=7, bpstype="linear", xmin=0.0, xmax=50.0, xsize=103, continuity="zero",
                      quad_order_additional=0, projection_algorithm=0),
        "vanilla": dict(order=5, bpstype="linear", xmin=0.0, xmax=10.0, xsize=12, continuity="vanilla",
                        quad_order_additional=2, projection_algorithm=0),
        "custom": dict(order=9, bpstype="linear", xmin=0.0, xmax=37.5, xsize=20, continuity="custom",
                       left_point_continuity=0, right_point_continuity=1, quad_order_additional=0,
                       projection_algorithm=0),
        "explinear": dict(order=7, bpstype="exponentiallinear", xmin=0.0, xmax=400.0, xsize=60, xpartition=20.0,
                          gamma=2.0, continuity="zero", quad_order_additional=0, projection_algorithm=0),
    }
    for name, kw in cases.items():
        b = ns["BSPLINE"]()
        b.ApplyConfigSection(_Conf(**kw))
        out["bs_%s_bp" % name] = b.GetBreakpointSequence().copy()
        out["bs_%s_cont" % name] = b.GetContinuitySequence().copy()
        out["bs_%s_knots" % name] = b.GetKnotSequence().copy()
        out["bs_%s_count" % name] = np.array(b.NumberOfBSplines)
        out["bs_%s_grid" % name] = b.GetQuadratureGridGlobal().copy()
        out["bs_%s_gw" % name] = b.GetQuadratureWeightsGlobal().copy()
        for k, v in kw.items():
            out["bs_%s_cfg_%s" % (name, k)] = np.array(v)
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, len(out), "arrays")


GEO_OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "geometry_golden.npz")
BANDNH_CASES = ((9, 2), (20, 6), (103, 6), (5, 6), (1, 0))
SELECTION_CASES = ((3, 0), (9, 0), (63, 0), (5, 2), (1, 0))


def geometry():
    ns = {"__name__": "pyprop_ref_geometry", "xrange": range}
    exec("from numpy import *", ns)
    for rel in (("tensorpotential", "GeometryInfo.py"), ("tensorpotential", "basis", "ReducedSphericalHarmonic.py")):
        path = os.path.join(REF, "pyprop", *rel)
        with open(path) as f:
            exec(compile(_py2_to_py3(f.read()), path, "exec"), ns)

    class _Tools:
        """Stand-in for core.ReducedSphericalTools: only GetSize() is used by the pair generator."""

        def __init__(self, lmax, m):
            self.lmax, self.m = lmax, m

        def GetSize(self):
            return self.lmax - abs(self.m)

    out = {}
    for n, k in BANDNH_CASES:
        g = ns["GeometryInfoCommonBandedNonHermitian"](n, k, False)
        out["bandnh_pairs_%d_%d" % (n, k)] = np.asarray(g.GetBasisPairs())
    for lmax, m in SELECTION_CASES:
        g = ns["GeometryInfoReducedSphHarmSelectionRule"](_Tools(lmax, m), False)
        out["selection_pairs_%d_%d" % (lmax, m)] = np.asarray(g.GetBasisPairs())
        out["selection_count_%d_%d" % (lmax, m)] = np.array(g.GetGlobalBasisPairCount())
    np.savez_compressed(GEO_OUT, **out)
    print("wrote", GEO_OUT, len(out), "arrays")


LASER_OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "laser_golden.npz")


def laser():
    """LaserFunctionVelocity of examples/tensor/helium_stabilization_sae/example.py:220-230, its
    source text cut out of the script (the rest is Python 2 and needs the compiled core), on a
    time grid that includes the pulse edges, with and without the optional phase key."""
    path = os.path.join(REF, "examples", "tensor", "helium_stabilization_sae", "example.py")
    src = open(path).read()
    m = re.search(r"^def LaserFunctionVelocity\(.*?(?=^\S)", src, flags=re.M | re.S)
    ns = {}
    exec("from numpy import *", ns)
    exec(compile(m.group(0), path, "exec"), ns)
    out = {}
    for name, kw in (("nophase", dict(amplitude=0.877, frequency=0.057, pulse_duration=8 * 2 * np.pi / 0.057)),
                     ("phase", dict(amplitude=1.754, frequency=0.057, pulse_duration=20 * 2 * np.pi / 0.057,
                                    phase=0.3))):
        T = kw["pulse_duration"]
        t = np.concatenate([[-1.0, 0.0, T * (1 - 1e-12), T, T + 1.0], np.linspace(0.0, T, 97)])
        out["laser_%s_t" % name] = t
        out["laser_%s_f" % name] = np.array([ns["LaserFunctionVelocity"](_Conf(**kw), x) for x in t])
        for k, v in kw.items():
            out["laser_%s_cfg_%s" % (name, k)] = np.array(v)
    np.savez_compressed(LASER_OUT, **out)
    print("wrote", LASER_OUT, len(out), "arrays")


if __name__ == "__main__":
    if not os.path.isdir(REF):
        sys.exit("reference tree not present; the committed fixture is used as is")
    main()
    geometry()
    laser()
