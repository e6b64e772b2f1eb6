"""Test infrastructure (the oracle), not product code.

Build recipe for the two CPU checkers, one shared library per model
configuration (precision, stepper, observer, sizes, model source):

* the *port*: ``clode_oracle.c``, this project's C restatement of clODE's
  ensemble kernels, built into ``oracle/_build/``;
* the *reference*: clODE's own OpenCL-C kernel sources
  (clode/cpp/{transient,initializeObserver,features,trajectory}.cl), compiled
  in place as C11 through ``ref_shim.h``/``ref_driver.c`` into
  ``oracle/_ref/``.  Only possible where the clODE source tree is present
  (``CLODE_REFERENCE_ROOT``; without it, a clODE checkout named
  ``reference`` beside this repository's root directory).

Both are compiled with ``-ffp-contract=off`` so that no multiply-add is fused
behind the reference's back, and with OpenMP over members when the compiler
supports it.  The -D set mirrors clode/cpp/CLODE.cpp:118-138 and
clode/cpp/CLODEfeatures.cpp:37-38.
"""
from __future__ import annotations

import hashlib
import os
import shutil
import subprocess
import tempfile
from dataclasses import dataclass, field

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_DIR = os.path.join(HERE, "_build")
REF_DIR = os.path.join(HERE, "_ref")
REFERENCE_ROOT = os.environ.get("CLODE_REFERENCE_ROOT",
                                os.path.normpath(os.path.join(HERE, os.pardir, os.pardir, "reference")))
REFERENCE_KERNEL_DIR = os.path.join(REFERENCE_ROOT, "clode", "cpp")

# stepper name -> define, clode/cpp/steppers.cl:26-43
STEPPER_DEFINES = {
    "euler": "EXPLICIT_EULER",
    "heun": "EXPLICIT_HEUN",
    "rk4": "EXPLICIT_RK4",
    "bs23": "EXPLICIT_BS23",
    "dopri5": "EXPLICIT_DOPRI5",
    "seuler": "STOCHASTIC_EULER",
}

# observer name -> define, clode/cpp/observers.cl:122-143 and each getObserverInfo_*
OBSERVER_DEFINES = {
    "basic": "USE_OBSERVER_BASIC",
    "basicall": "USE_OBSERVER_BASIC_ALLVAR",
    "localmax": "USE_OBSERVER_LOCAL_MAX",
    "nhood1": "USE_OBSERVER_NEIGHBORHOOD_1",
    "nhood2": "USE_OBSERVER_NEIGHBORHOOD_2",
    "thresh2": "USE_OBSERVER_THRESHOLD_2",
}

CFLAGS = ["-O3", "-std=gnu11", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math", "-w"]


@dataclass(frozen=True)
class OracleConfig:
    rhs_file: str
    n_var: int
    n_par: int
    n_aux: int = 0
    n_wiener: int = 0
    stepper: str = "rk4"
    single_precision: bool = False
    observer: str | None = None
    n_store_events: int = 0
    extra: tuple = field(default_factory=tuple)

    def defines(self) -> list[str]:
        d = [
            "-DCLODE_SINGLE_PRECISION" if self.single_precision else "-DCLODE_DOUBLE_PRECISION",
            "-D" + STEPPER_DEFINES[self.stepper],
            f"-DN_PAR={self.n_par}",
            f"-DN_VAR={self.n_var}",
            f"-DN_AUX={self.n_aux}",
            f"-DN_WIENER={self.n_wiener}",
            f"-DN_STORE_EVENTS={self.n_store_events}",
        ]
        if self.observer is not None:
            d += ["-D" + OBSERVER_DEFINES[self.observer], "-DCLODE_WITH_OBSERVER"]
        return d + list(self.extra)


_OPENMP_OK: bool | None = None


def _openmp_supported() -> bool:
    global _OPENMP_OK
    if _OPENMP_OK is None:
        with tempfile.TemporaryDirectory() as td:
            src = os.path.join(td, "t.c")
            with open(src, "w") as f:
                f.write("#include <omp.h>\nint f(void){return omp_get_max_threads();}\n")
            r = subprocess.run(["gcc", "-fopenmp", "-fPIC", "-shared", src, "-o", os.path.join(td, "t.so")],
                               capture_output=True)
            _OPENMP_OK = r.returncode == 0
    return _OPENMP_OK


def _digest(parts: list[str], files: list[str]) -> str:
    h = hashlib.sha256()
    for p in parts:
        h.update(p.encode())
        h.update(b"\0")
    for fn in files:
        with open(fn, "rb") as f:
            h.update(f.read())
    return h.hexdigest()[:20]


def _compile(out_dir: str, tag: str, sources: list[str], include_dirs: list[str], cfg: OracleConfig,
             dep_files: list[str]) -> str:
    os.makedirs(out_dir, exist_ok=True)
    rhs = os.path.abspath(cfg.rhs_file)
    flags = CFLAGS + (["-fopenmp"] if _openmp_supported() else [])
    key = _digest(flags + cfg.defines() + sources + include_dirs, dep_files + [rhs])
    out = os.path.join(out_dir, f"{tag}_{key}.so")
    if os.path.exists(out):
        return out
    cmd = ["gcc"] + flags + [f"-I{d}" for d in include_dirs] + cfg.defines()
    cmd += [f'-DCLODE_RHS_FILE="{rhs}"'] + sources
    tmp = out + f".tmp{os.getpid()}"
    cmd += ["-o", tmp, "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed ({tag}):\n{' '.join(cmd)}\n{r.stderr}")
    os.replace(tmp, out)
    return out


def build_port(cfg: OracleConfig) -> str:
    """Compile this project's C restatement for ``cfg``; returns the .so path."""
    src = os.path.join(HERE, "clode_oracle.c")
    return _compile(PORT_DIR, "port", [src], [HERE], cfg, [src, os.path.join(HERE, "port_shim.h")])


def reference_available() -> bool:
    return os.path.isfile(os.path.join(REFERENCE_KERNEL_DIR, "transient.cl")) and shutil.which("gcc") is not None


def build_reference(cfg: OracleConfig) -> str:
    """Compile clODE's own kernel sources (read in place) for ``cfg``."""
    if not reference_available():
        raise FileNotFoundError(f"clODE sources not found under {REFERENCE_ROOT}")
    drv = os.path.join(HERE, "ref_driver.c")
    deps = [drv, os.path.join(HERE, "ref_shim.h")]
    for fn in sorted(os.listdir(REFERENCE_KERNEL_DIR)):
        if fn.endswith(".cl"):
            deps.append(os.path.join(REFERENCE_KERNEL_DIR, fn))
    for sub in ("steppers", "observers"):
        d = os.path.join(REFERENCE_KERNEL_DIR, sub)
        deps += [os.path.join(d, fn) for fn in sorted(os.listdir(d)) if fn.endswith(".clh")]
    return _compile(REF_DIR, "ref", [drv], [HERE, REFERENCE_KERNEL_DIR], cfg, deps)
