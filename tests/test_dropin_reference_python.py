"""clODE's own Python package on top of this engine's module.

clODE's front-end (``clode/solver.py``, ``features.py``, ``trajectory.py``,
``runtime.py``, ``__init__.py``) imports its compiled module as
``clode.cpp.clode_cpp_wrapper``.  This test reads those files where the clODE
source tree exists (CLODE_REFERENCE_ROOT, else a checkout named ``reference``
beside this repository; skipped elsewhere) and checks that
``clode_gb300.clode_cpp_wrapper`` can stand in for that module:

* every name they import from the module exists;
* every call they make on the module's objects — the simulator held in
  ``self._integrator`` (``SimulatorBase`` in solver.py, ``FeatureSimulatorBase``
  in features.py, ``TrajectorySimulatorBase`` in trajectory.py), the problem,
  solver and observer parameter objects (``self._pi``, ``self._sp``,
  ``self._op``), the device resource (``self._runtime``), the logger
  (``get_logger()``) and the module's own classes and functions — names an
  existing attribute and binds to its signature with the same positional
  arguments and keywords;
* every attribute they read or write on those objects exists;
* clODE's own ``FeatureSimulator`` and ``TrajectorySimulator``, imported
  with the module substituted, construct up to device creation (on a machine
  without a GPU that is where the engine reports the missing device).
"""
import ast
import inspect
import os
import sys

import pytest

from oracle.build import REFERENCE_ROOT

PKG = os.path.join(REFERENCE_ROOT, "clode")
FILES = ("solver.py", "features.py", "trajectory.py", "runtime.py", "__init__.py")
MODULE = "clode.cpp.clode_cpp_wrapper"

pytestmark = pytest.mark.skipif(not os.path.isfile(os.path.join(PKG, "solver.py")),
                                reason="clODE's Python sources are not present")

# the class of self._integrator in each file (clode/solver.py:208, features.py:376, trajectory.py:158)
INTEGRATOR = {"solver.py": "SimulatorBase", "features.py": "FeatureSimulatorBase",
              "trajectory.py": "TrajectorySimulatorBase"}
# other objects of the module held by clODE's front-end classes
HELD = {"_pi": "ProblemInfo", "_sp": "SolverParams", "_op": "ObserverParams", "_runtime": "OpenCLResource"}


def _wrapper():
    from clode_gb300 import clode_cpp_wrapper as W
    return W


def _tree(name):
    with open(os.path.join(PKG, name)) as f:
        return ast.parse(f.read(), filename=name)


def _imported_names(tree):
    names = set()
    for node in ast.walk(tree):
        if isinstance(node, ast.ImportFrom) and node.module == MODULE:
            names.update(a.name for a in node.names)
    return names


def _receiver(node, fname, imported):
    """Name of the module class an expression refers to an instance of, or
    ('module', name) for the module's own names, else None."""
    if isinstance(node, ast.Attribute) and isinstance(node.value, ast.Name) and node.value.id == "self":
        if node.attr == "_integrator" and fname in INTEGRATOR:
            return INTEGRATOR[fname]
        return HELD.get(node.attr)
    if isinstance(node, ast.Call) and isinstance(node.func, ast.Name) and node.func.id == "get_logger":
        return "<logger>"
    if isinstance(node, ast.Name) and node.id in imported:
        return ("module", node.id)
    return None


def _resolve(W, rec):
    if rec == "<logger>":
        return type(W.get_logger())
    if isinstance(rec, tuple):
        return getattr(W, rec[1])
    return getattr(W, rec)


def _uses(fname):
    """(kind, receiver, attribute, n_positional, keywords, line) for every use."""
    tree = _tree(fname)
    imported = _imported_names(tree)
    out = []
    calls = set()
    for node in ast.walk(tree):
        if isinstance(node, ast.Call):
            f = node.func
            has_star = any(isinstance(a, ast.Starred) for a in node.args) or any(k.arg is None for k in node.keywords)
            kws = tuple(k.arg for k in node.keywords if k.arg is not None)
            if isinstance(f, ast.Attribute):
                rec = _receiver(f.value, fname, imported)
                if rec is not None:
                    out.append(("call", rec, f.attr, len(node.args), kws, has_star, node.lineno))
                    calls.add(id(f))
            elif isinstance(f, ast.Name) and f.id in imported:
                out.append(("call", ("module", f.id), None, len(node.args), kws, has_star, node.lineno))
    for node in ast.walk(tree):
        if isinstance(node, ast.Attribute) and id(node) not in calls:
            rec = _receiver(node.value, fname, imported)
            if rec is not None:
                out.append(("attr", rec, node.attr, 0, (), False, node.lineno))
    return imported, out


def _bind(obj, n_pos, kws, bound_method):
    sig = inspect.signature(obj)
    params = list(sig.parameters.values())
    if bound_method and params and params[0].name == "self":
        params = params[1:]
    sig = sig.replace(parameters=params)
    sig.bind(*([None] * n_pos), **{k: None for k in kws})


@pytest.mark.parametrize("fname", FILES)
def test_every_imported_name_exists(fname):
    W = _wrapper()
    missing = sorted(n for n in _imported_names(_tree(fname)) if not hasattr(W, n))
    assert not missing, f"{fname} imports {missing} from {MODULE}"


@pytest.mark.parametrize("fname", FILES)
def test_every_call_and_attribute_is_compatible(fname):
    W = _wrapper()
    _, uses = _uses(fname)
    problems = []
    checked = 0
    for kind, rec, attr, n_pos, kws, has_star, line in uses:
        cls = _resolve(W, rec)
        where = f"{fname}:{line}"
        if kind == "attr":
            if isinstance(rec, tuple):
                ok = hasattr(cls, attr)
            else:
                ok = hasattr(cls, attr) or attr in _instance_attributes(W, cls)
            if not ok:
                problems.append(f"{where}: {cls.__name__} has no attribute {attr!r}")
            checked += 1
            continue
        target = cls if attr is None else getattr(cls, attr, None)
        if target is None:
            problems.append(f"{where}: {cls.__name__} has no method {attr!r}")
            continue
        if has_star:
            checked += 1
            continue
        try:
            if inspect.isclass(target):
                _bind(target.__init__, n_pos, kws, bound_method=True)
            else:
                _bind(target, n_pos, kws, bound_method=attr is not None and not isinstance(
                    inspect.getattr_static(cls, attr), (staticmethod, classmethod)))
        except TypeError as e:
            problems.append(f"{where}: {getattr(target, '__qualname__', target)}"
                            f"({n_pos} positional, keywords {list(kws)}): {e}")
        checked += 1
    assert not problems, "\n".join(problems)
    if fname in INTEGRATOR:
        assert checked > 5  # the walk found the simulator calls


_INSTANCE_ATTRS = {}


def _instance_attributes(W, cls):
    """Attributes set on instances of the module's value classes (the
    parameter structs keep their fields as instance attributes)."""
    if cls not in _INSTANCE_ATTRS:
        try:
            if cls is W.ProblemInfo:
                obj = cls("m.cl", ["x"], ["p"], [], 0)
            else:
                obj = cls()
            _INSTANCE_ATTRS[cls] = set(vars(obj))
        except Exception:
            _INSTANCE_ATTRS[cls] = set()
    return _INSTANCE_ATTRS[cls]


def _import_reference_package(monkeypatch):
    W = _wrapper()
    for k in [k for k in sys.modules if k == "clode" or k.startswith("clode.")]:
        monkeypatch.delitem(sys.modules, k)
    monkeypatch.setitem(sys.modules, MODULE, W)
    monkeypatch.syspath_prepend(REFERENCE_ROOT)
    import importlib
    import warnings
    with warnings.catch_warnings():
        warnings.simplefilter("ignore", SyntaxWarning)  # escape sequences in clode/xpp_parser.py
        clode = importlib.import_module("clode")
    assert os.path.dirname(clode.__file__) == os.path.normpath(PKG)
    return clode, W


def _device_count():
    import ctypes as C
    from clode_gb300 import _native as N
    n = C.c_int(0)
    return n.value if N.lib.clode_device_count(C.byref(n)) == 0 else 0


@pytest.mark.parametrize("kind", ["features", "trajectory"])
def test_reference_front_end_constructs_up_to_the_device(monkeypatch, kind):
    clode, W = _import_reference_package(monkeypatch)
    from clode_gb300 import rhs_path
    common = dict(src_file=rhs_path("lactotroph.cl"), variables={"v": -60.0, "n": 0.0, "f": 0.0, "c": 0.1},
                  parameters={"gcal": 1.0, "gsk": 3.0, "gbk": 1.0}, aux=["ica"], stepper=clode.Stepper.dormand_prince,
                  t_span=(0.0, 100.0))
    try:
        if kind == "features":
            sim = clode.FeatureSimulator(observer=clode.Observer.neighbourhood_2, event_var="c", feature_var="v",
                                         **common)
        else:
            sim = clode.TrajectorySimulator(**common)
    except RuntimeError as e:
        # no GPU on this machine: construction got as far as the device
        assert "no CUDA device" in str(e)
        assert _device_count() == 0
        return
    # with a GPU the simulator is built and usable through clODE's own API
    assert sim.variable_names == ["v", "n", "f", "c"]
