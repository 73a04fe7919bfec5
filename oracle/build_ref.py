"""Build the reference's own CPU implementation of the sparse-PCA path.

Test and baseline infrastructure only: the product never imports it.

Two stages, both writing only under ``oracle/_ref/`` (git-ignored):

1. ``cythonize`` (needs Cython and the reference checkout): translate the
   reference modules on the path -- ``brisc/cyutils.pyx``, ``brisc/pca.pyx``,
   ``brisc/normalize.pyx``, ``brisc/cysparse.pyx``, ``brisc/hvg.pyx``,
   ``brisc/kmeans.pyx``, ``brisc/knn.pyx``, ``brisc/harmonize.pyx`` -- plus
   the test harness
   ``oracle/ref_probe.pyx`` to C++ under ``oracle/_ref/gen/``. The sources are
   read where they lie; nothing is copied into the repository.
2. ``compile`` (needs only g++, Python and numpy headers): build every
   ``oracle/_ref/gen/*.cpp`` into ``oracle/_ref/<machine>/brisc/*.so`` with the
   reference's own Linux flags (``setup.py:92-100`` of the reference:
   ``-Ofast -funroll-loops -std=c++17 -fopenmp`` plus the ``-march`` of the
   variant the reference would load on this CPU, ``setup.py:34-42`` and
   ``brisc/utils.py:29-49``: on aarch64 the SVE build only where numpy
   reports SVE. The GPU host's Grace cores list no ``sve`` in
   ``/proc/cpuinfo`` and numpy reports none there, so the reference itself
   loads its plain ``armv8.2-a`` build on that host, and so does this recipe).

Stage 2 runs on any machine that received ``oracle/_ref/gen`` (the C++ is
architecture-neutral), so the aarch64 GPU host can rebuild the reference
without Cython.

Usage::

    python oracle/build_ref.py [--reference DIR] [--jobs N] [--compile-only]
"""
from __future__ import annotations

import argparse
import os
import platform
import subprocess
import sys
import sysconfig
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
REF_OUT = HERE / "_ref"
GEN = REF_OUT / "gen"
MODULES = ["cyutils", "pca", "normalize", "cysparse", "hvg", "kmeans", "knn",
           "harmonize", "hdf5"]
# What the CPU baselines need (cysparse's 24 MB of C++ is only needed for the
# transpose fixture and is skipped where compile time matters).
BASELINE_MODULES = ["cyutils", "pca", "normalize", "hvg", "kmeans", "knn",
                    "harmonize", "hdf5", "ref_probe"]
DIRECTIVES = {"language_level": "3", "boundscheck": False,
              "wraparound": False, "cdivision": True,
              "initializedcheck": False, "warn.undeclared": False}


def reference_dir() -> Path:
    """The reference checkout this recipe reads: $BRISC_REFERENCE, else the
    container's read-only mount. Absent on machines that only compile."""
    return Path(os.environ.get("BRISC_REFERENCE", "/root/reference"))


def have_reference() -> bool:
    return (reference_dir() / "brisc" / "pca.pyx").exists()


def machine_dir() -> Path:
    return REF_OUT / platform.machine().lower()


def march_flag() -> list[str]:
    """The -march of the variant the reference itself would load here: its
    setup.py:34-42 builds one per instruction-set level and its
    import_cython (brisc/utils.py:29-49) picks x86-64-v4 with AVX-512F, v3
    with AVX2, else v2; on aarch64 the SVE build where numpy reports SVE,
    else plain armv8.2-a."""
    m = platform.machine().lower()
    try:
        from numpy._core._multiarray_umath import __cpu_features__ as cpu
    except ImportError:
        cpu = {}
    if m in ("x86_64", "amd64"):
        return ["-march=x86-64-v4" if cpu.get("AVX512F") else
                "-march=x86-64-v3" if cpu.get("AVX2") else "-march=x86-64-v2"]
    if m == "aarch64":
        return ["-march=armv8.2-a+sve" if cpu.get("SVE") else "-march=armv8.2-a"]
    return []


def cythonize(reference: Path) -> None:
    from Cython.Compiler.Main import CompilationOptions, compile_single
    GEN.mkdir(parents=True, exist_ok=True)
    jobs = [(reference / "brisc" / f"{m}.pyx", GEN / f"brisc.{m}.cpp")
            for m in MODULES]
    jobs.append((HERE / "ref_probe.pyx", GEN / "brisc.ref_probe.cpp"))
    for src, out in jobs:
        if out.exists() and out.stat().st_mtime >= src.stat().st_mtime:
            continue
        opts = CompilationOptions(
            cplus=True, output_file=str(out), language_level=3,
            include_path=[str(reference)], compiler_directives=DIRECTIVES)
        if src.parent == HERE:
            # The harness is compiled as the module `brisc.ref_probe`.
            opts.module_name = "brisc.ref_probe"
        res = compile_single(str(src), opts,
                             full_module_name="brisc." + src.stem)
        if res.num_errors:
            raise RuntimeError(f"cython failed on {src}")
        # progress on stderr: stdout of a bench run is its one JSON line
        print(f"cythonized {src.name} -> {out.relative_to(HERE)}", file=sys.stderr)


def compile_all(jobs: int, modules: list[str] | None = None) -> Path:
    import numpy as np
    out_pkg = machine_dir() / "brisc"
    out_pkg.mkdir(parents=True, exist_ok=True)
    (out_pkg / "__init__.py").write_text("")
    ext = sysconfig.get_config_var("EXT_SUFFIX") or ".so"
    inc = [sysconfig.get_paths()["include"], np.get_include()]
    flags = ["-Ofast", "-funroll-loops", "-std=c++17", "-g0", "-fopenmp",
             "-fPIC", "-shared", "-w",
             "-DNPY_NO_DEPRECATED_API=NPY_1_17_API_VERSION",
             *march_flag(), *[f"-I{i}" for i in inc]]
    cpps = sorted(GEN.glob("brisc.*.cpp"))
    if modules is not None:
        cpps = [c for c in cpps if c.stem.split(".", 1)[1] in modules]
    if not cpps:
        raise FileNotFoundError(
            f"no generated C++ under {GEN}; run the cythonize stage where "
            "the reference checkout and Cython are available")

    # the flags of the last build: a different -march rebuilds everything
    stamp = machine_dir() / "flags.txt"
    same_flags = stamp.exists() and stamp.read_text() == " ".join(flags)

    def one(cpp: Path) -> str:
        mod = cpp.stem.split(".", 1)[1]
        so = out_pkg / f"{mod}{ext}"
        if same_flags and so.exists() and so.stat().st_mtime >= cpp.stat().st_mtime:
            return f"up to date {so.name}"
        cmd = ["g++", *flags, str(cpp), "-o", str(so), "-fopenmp"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError(f"g++ failed on {cpp.name}:\n{r.stderr[-4000:]}")
        return f"built {so.relative_to(HERE)}"

    with ThreadPoolExecutor(max_workers=jobs) as ex:
        for msg in ex.map(one, cpps):
            print(msg, file=sys.stderr)
    stamp.write_text(" ".join(flags))
    return machine_dir()


def built_march() -> str:
    """The -march the compiled reference modules here were built with."""
    stamp = machine_dir() / "flags.txt"
    if not stamp.exists():
        return "unknown"
    return next((f for f in stamp.read_text().split() if f.startswith("-march")),
                "default")


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--reference", default=str(reference_dir()))
    ap.add_argument("--jobs", type=int, default=os.cpu_count() or 4)
    ap.add_argument("--compile-only", action="store_true")
    ap.add_argument("--baseline-only", action="store_true",
                    help="compile only the modules the CPU baseline needs")
    a = ap.parse_args(argv)
    ref = Path(a.reference)
    if not a.compile_only and (ref / "brisc" / "pca.pyx").exists():
        cythonize(ref)
    compile_all(a.jobs, BASELINE_MODULES if a.baseline_only else None)
    return 0


if __name__ == "__main__":
    sys.exit(main())
