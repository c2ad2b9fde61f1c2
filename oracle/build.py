"""Build recipes of the checker (test infrastructure, not the product).

* ``build_oracle()`` compiles the C restatement of the shader path (``sppm_oracle.c``) twice --
  single precision and double precision -- into ``oracle/_build/``.
* ``build_ref(reference_dir)`` compiles the reference's own sources from a reference checkout into
  ``oracle/_ref/``.  The checkout is the ``reference_dir`` argument, else the ``SPPM_REFERENCE_DIR``
  environment variable; with neither, nothing is built and a message says why.  The directory a
  build used is recorded in ``oracle/_ref/REFERENCE_DIR`` so that later test runs find the same
  sources (``reference_dir()``):
    - ``ref_host_dump``: the reference's ``mesh.cpp``, ``bvh.cpp``, ``bbox.cpp`` and ``camera.cpp``,
      unmodified, linked with ``ref_host_dump.cpp``;
    - ``libref_shaders.so``: the reference's GLSL shaders compiled as C++ through
      ``glsl_compat.hpp`` (see ``ref_shaders.cpp``).
  The sources are read where they lie; nothing of the reference is copied into the repository.
  ``oracle/_ref/`` is git-ignored.

All host code is compiled with ``-ffp-contract=off`` and without fast-math so that every
single-precision operation rounds exactly as written, on x86-64 and on aarch64 alike.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

ORACLE_DIR = Path(__file__).resolve().parent
REPO = ORACLE_DIR.parent
BUILD_DIR = ORACLE_DIR / "_build"
REF_DIR = ORACLE_DIR / "_ref"
INCLUDE = REPO / "include"
_RECORDED = REF_DIR / "REFERENCE_DIR"

STRICT_FP = ["-ffp-contract=off", "-fno-fast-math"]

# a GLSL floating literal (single precision): digits with a point and/or an exponent
_FLOAT_LITERAL = __import__("re").compile(
    r"(?<![\w.])((?:\d+\.\d*|\.\d+)(?:[eE][+-]?\d+)?|\d+[eE][+-]?\d+)(?![\w.])")


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"command failed ({proc.returncode}): {' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")


def _stale(target: Path, sources: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(s.stat().st_mtime > t for s in sources)


def build_oracle(force: bool = False) -> dict[str, Path]:
    """Compile the FP32 and FP64 oracles; returns {"f32": path, "f64": path}."""
    BUILD_DIR.mkdir(parents=True, exist_ok=True)
    src = ORACLE_DIR / "sppm_oracle.c"
    deps = [src, INCLUDE / "sppm.h", INCLUDE / "sppm_fpmath.h"]
    out = {}
    for tag, extra in (("f32", []), ("f64", ["-DORACLE_FP64"])):
        lib = BUILD_DIR / f"liboracle_{tag}.so"
        if force or _stale(lib, deps):
            tmp = lib.with_suffix(f".so.tmp{os.getpid()}")
            _run(["gcc", "-std=gnu11", "-O2", "-fopenmp", *STRICT_FP, "-fPIC", "-shared",
                  "-fvisibility=hidden", *extra, f"-I{INCLUDE}", str(src), "-o", str(tmp), "-lm"])
            os.replace(tmp, lib)
        out[tag] = lib
    return out


def _is_checkout(d: Path | None) -> bool:
    return d is not None and (d / "bvh.cpp").is_file() and (d / "photontrace.fs").is_file()


def reference_dir() -> Path | None:
    """The reference checkout: SPPM_REFERENCE_DIR, else the one the last build_ref() used, else None."""
    env = os.environ.get("SPPM_REFERENCE_DIR")
    if env:
        return Path(env)
    if _RECORDED.is_file():
        return Path(_RECORDED.read_text().strip())
    return None


def reference_available() -> bool:
    return _is_checkout(reference_dir())


def build_ref(reference_dir_: str | Path | None = None, force: bool = False) -> dict[str, Path]:
    """Compile the reference's host code and shaders into oracle/_ref (needs a reference checkout)."""
    src = Path(reference_dir_) if reference_dir_ else (Path(os.environ["SPPM_REFERENCE_DIR"])
                                                     if os.environ.get("SPPM_REFERENCE_DIR") else None)
    if src is None:
        print("oracle/build.py: no reference checkout given (argument or SPPM_REFERENCE_DIR); "
              "oracle/_ref is not built and the reference-marked tests will skip")
        return {}
    if not _is_checkout(src):
        print(f"oracle/build.py: {src} is not a glslppm checkout (bvh.cpp, photontrace.fs); oracle/_ref is not built")
        return {}
    REFERENCE = src.resolve()
    REF_DIR.mkdir(parents=True, exist_ok=True)
    _RECORDED.write_text(str(REFERENCE) + "\n")
    out = {}
    host_srcs = [REFERENCE / f for f in ("mesh.cpp", "bvh.cpp", "bbox.cpp", "camera.cpp")]
    dump = REF_DIR / "ref_host_dump"
    dump_src = ORACLE_DIR / "ref_host_dump.cpp"
    if force or _stale(dump, host_srcs + [dump_src]):
        _run(["g++", "-std=c++14", "-O2", *STRICT_FP, "-w", f"-I{REFERENCE}", str(dump_src),
              *map(str, host_srcs), "-o", str(dump)])
    out["host_dump"] = dump
    # the drop-in header include/sppm_gpurt.hpp compiled into the reference's own host code
    shim = REF_DIR / "ref_gpurt_shim_test"
    shim_src = ORACLE_DIR / "ref_gpurt_shim_test.cpp"
    native_lib = REPO / "glslppm_gb300" / "_lib" / "libsppm.so"
    if native_lib.exists() and (force or _stale(shim, host_srcs + [shim_src, INCLUDE / "sppm_gpurt.hpp", native_lib])):
        _run(["g++", "-std=c++14", "-O2", *STRICT_FP, "-w", f"-I{REFERENCE}", f"-I{INCLUDE}", str(shim_src),
              *map(str, host_srcs), f"-L{native_lib.parent}", "-lsppm", f"-Wl,-rpath,{native_lib.parent}",
              "-o", str(shim)])
    if shim.exists():
        out["gpurt_shim"] = shim
    shader_src = ORACLE_DIR / "ref_shaders.cpp"
    if shader_src.exists():
        compat = ORACLE_DIR / "glsl_compat.hpp"
        lib = REF_DIR / "libref_shaders.so"
        shaders = [REFERENCE / f for f in ("eyeraytrace.fs", "photontrace.fs", "hash.fs", "progressive.fs",
                                           "scatter.vs", "correction.vs", "re.fs", "min.fs", "max.fs", "sum.fs")]
        if force or _stale(lib, shaders + [shader_src, compat, INCLUDE / "sppm_fpmath.h"]):
            # each shader body (the source without its '#version' line) is placed in its own
            # namespace by ref_shaders.cpp; the bodies are produced into oracle/_ref only
            for sh in shaders:
                body = REF_DIR / (sh.name.replace(".", "_") + ".inc")
                lines = sh.read_text(encoding="latin-1").splitlines(keepends=True)
                text = "".join(l if not l.lstrip().startswith("#version") else "\n" for l in lines)
                body.write_text(_FLOAT_LITERAL.sub(lambda m: m.group(1) + "f", text), encoding="latin-1")
            _run(["g++", "-std=c++17", "-O2", *STRICT_FP, "-fPIC", "-shared", "-fvisibility=hidden", "-w",
                  f"-I{INCLUDE}", f"-I{ORACLE_DIR}", f"-I{REF_DIR}", str(shader_src), "-o", str(lib)])
        out["shaders"] = lib
    return out


def clean() -> None:
    for d in (BUILD_DIR, REF_DIR):
        if d.exists():
            shutil.rmtree(d)


if __name__ == "__main__":
    import sys
    print(build_oracle(force=True))
    print(build_ref(sys.argv[1] if len(sys.argv) > 1 else None, force=True))
