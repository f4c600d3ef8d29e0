"""TEST INFRASTRUCTURE ONLY: builds the CPU oracle libraries.

- oracle/_build/liboracle.so: the plain-C restatement (oracle.c + sw_extra.c).
  Builds anywhere from this repository alone.
- oracle/_ref/libref_L<L>_T<T>.so: the reference's own task sources compiled
  unmodified, where they lie under the reference checkout, against the header
  shim in oracle/shim/, plus ref_driver.cc.  Beside the checkout
  (MPASO_REFERENCE_DIR, default /root/reference) each translation unit is
  first amalgamated with the headers it includes into oracle/_ref/refsrc/;
  the libraries are compiled from those units, which also lets a host without
  the checkout build them.  All outputs are git-ignored.

Usage: python oracle/build.py [--force]
"""
import os
import platform
import re
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("MPASO_REFERENCE_DIR", "/root/reference")
CFLAGS = ["-O3", "-fPIC", "-ffp-contract=off", "-fno-fast-math"]
REF_SOURCES = ["apps/sw/tasks/solve.cc", "apps/ocean/tasks/solve.cc",
               "apps/ocean/tasks/init_functions.cc"]
# (levels, tracers) of the reference builds used by the pin tests.
REF_CONFIGS = [(1, 1), (3, 2), (5, 5)]
GRAVITY = "9.80616"  # mpasoflecsi/common/constants.hh:30-31


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + " ".join(cmd) + "\n" + r.stderr)


def _foreign(path):
    """Whether the ELF file `path` was built for another machine than this host's."""
    want = {"x86_64": 62, "aarch64": 183}.get(platform.machine())
    with open(path, "rb") as f:
        hdr = f.read(20)
    return want is not None and hdr[:4] == b"\x7fELF" and int.from_bytes(hdr[18:20], "little") != want


def _stale(out, deps):
    if not os.path.exists(out) or _foreign(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build_restatement(force=False):
    out_dir = os.path.join(HERE, "_build")
    os.makedirs(out_dir, exist_ok=True)
    out = os.path.join(out_dir, "liboracle.so")
    deps = [os.path.join(HERE, f) for f in ("oracle.c", "sw_extra.c", "oracle.h", "build.py")]
    if force or _stale(out, deps):
        _run(["gcc", "-std=c11", *CFLAGS, "-shared", "-o", out, deps[0], deps[1], "-lm"])
    return out


def ref_available():
    return all(os.path.exists(os.path.join(REF, s)) for s in REF_SOURCES)


REF_UNIT_DIR = os.path.join(HERE, "_ref", "refsrc")  # the reference builds' translation units, amalgamated
REF_UNITS = [s.replace("/", "_") for s in REF_SOURCES] + ["ref_driver.cc"]


def ref_units():
    """Paths of the reference builds' translation units (REF_SOURCES and
    ref_driver.cc, each amalgamated with the shim and reference headers it
    includes), written beside the checkout; None where neither the checkout
    nor the units are present."""
    if ref_available():
        os.makedirs(REF_UNIT_DIR, exist_ok=True)
        srcs = [os.path.join(REF, s) for s in REF_SOURCES] + [os.path.join(HERE, "ref_driver.cc")]
        for name, src in zip(REF_UNITS, srcs):
            _write_if_changed(os.path.join(REF_UNIT_DIR, name), amalgamate(src, [os.path.join(HERE, "shim"), REF, HERE],
                                                                             _label))
    units = [os.path.join(REF_UNIT_DIR, n) for n in REF_UNITS]
    return units if all(os.path.exists(u) for u in units) else None


def build_ref(force=False):
    """Returns {(L, T): path} for the reference builds (empty without the
    checkout or its amalgamated units): the reference's task sources, compiled
    from the units, so a host without the checkout builds the same libraries
    from the units made beside one."""
    units = ref_units()
    if units is None:
        return {}
    out_dir = os.path.join(HERE, "_ref")
    deps = units + [os.path.join(HERE, f) for f in ("sw_extra.c", "oracle.h", "build.py")]

    def one(cfg):
        L, T = cfg
        out = os.path.join(out_dir, f"libref_L{L}_T{T}.so")
        if not (force or _stale(out, deps)):
            return cfg, out
        defs = [f"-DMPASO_REF_NVL={L}", f"-DMPASO_REF_NTR={T}", f"-DMPASO_REF_GRAVITY={GRAVITY}"]
        objs = []
        for u in units:
            obj = os.path.join(out_dir, f"L{L}_T{T}_" + os.path.basename(u) + ".o")
            _run(["g++", "-std=c++17", *CFLAGS, *defs, "-w", "-c", u, "-o", obj])
            objs.append(obj)
        obj = os.path.join(out_dir, f"L{L}_T{T}_sw_extra.o")
        _run(["gcc", "-std=c11", *CFLAGS, f"-I{HERE}", "-c", os.path.join(HERE, "sw_extra.c"), "-o", obj])
        objs.append(obj)
        _run(["g++", "-shared", "-o", out, *objs, "-lm"])
        return cfg, out

    with ThreadPoolExecutor(max_workers=len(REF_CONFIGS) + 1) as ex:
        cstep = ex.submit(build_cstep, force)
        out = dict(ex.map(one, REF_CONFIGS))
        out["cstep"] = cstep.result()
        return out


def _label(p):
    """Name of a file in the #line directives of an amalgamated unit."""
    p = os.path.realpath(p)
    for base, name in ((os.path.realpath(REF), "reference"), (os.path.realpath(os.path.dirname(HERE)), ".")):
        if p.startswith(base + os.sep):
            return os.path.join(name, os.path.relpath(p, base))
    return os.path.basename(p)


_INCLUDE = re.compile(r'^\s*#\s*include\s*([<"])([^>"]+)[>"]')
_ONCE = re.compile(r"^\s*#\s*pragma\s+once\b")


def amalgamate(src, dirs, label):
    """Text of the translation unit `src` with every #include that resolves in
    `dirs` (a quoted one first beside the including file, as the compiler looks)
    replaced by the included file's text, recursively; headers found nowhere in
    `dirs` (the system's) stay #include lines.  A header with #pragma once is
    inlined once; #line directives keep diagnostics pointing at the sources.
    `label(path)` names a file in those directives."""
    once, out = set(), []

    def emit(path):
        with open(path) as f:
            text = f.read().splitlines()
        if any(_ONCE.match(x) for x in text):
            real = os.path.realpath(path)
            if real in once:
                return
            once.add(real)
        out.append(f'#line 1 "{label(path)}"')
        for n, line in enumerate(text, 1):
            if _ONCE.match(line):
                out.append("")
                continue
            m = _INCLUDE.match(line)
            if m:
                look = ([os.path.dirname(path)] if m.group(1) == '"' else []) + list(dirs)
                hit = next((os.path.join(d, m.group(2)) for d in look if os.path.isfile(os.path.join(d, m.group(2)))),
                           None)
                if hit:
                    emit(hit)
                    out.append(f'#line {n + 1} "{label(path)}"')
                    continue
            out.append(line)

    emit(src)
    return "\n".join(out) + "\n"


FLW_DIR = os.path.join(HERE, "_ref", "flw")  # the wrapper build's translation units, amalgamated
FLW_UNITS = ["init_functions.cc", "ref_driver.cc", "flecsi_probe.cc", "sw_tasks.cc", "ocean_tasks.cc"]


def _write_if_changed(path, text):
    if os.path.exists(path):
        with open(path) as f:
            if f.read() == text:
                return
    with open(path, "w") as f:
        f.write(text)


def build_flecsi_wrappers(force=False):
    """oracle/_ref/libref_gb300_L1_T1.so: the reference's own driver logic
    (ref_driver.cc) and FCT setup (init_functions.cc) with the FleCSI wrapper
    library's task bodies (mpas-o-flecsi-2.0_gb300/flecsi/) in place of the
    reference's apps/sw/tasks/solve.cc and apps/ocean/tasks/solve.cc, linked
    against libmpaso: it links only if every task the driver calls is defined
    with the reference's declared signature.

    Two steps.  Where the reference checkout is present, each translation unit
    is amalgamated (its reference, shim and wrapper headers inlined) into
    oracle/_ref/flw/, a git-ignored build output like the libraries.  The
    units are then compiled from there, so a host without the checkout builds
    the library from the units made beside one.  None when
    neither the checkout nor the units are there."""
    pkg = os.path.join(os.path.dirname(HERE), "mpas-o-flecsi-2.0_gb300")
    wrap = os.path.join(pkg, "flecsi")
    lib_dir = os.path.join(pkg, "lib")
    out_dir = os.path.join(HERE, "_ref")
    root = os.path.dirname(HERE)
    if ref_available():
        os.makedirs(FLW_DIR, exist_ok=True)
        srcs = [os.path.join(REF, "apps/ocean/tasks/init_functions.cc"), os.path.join(HERE, "ref_driver.cc"),
                os.path.join(HERE, "flecsi_probe.cc"), os.path.join(wrap, "sw_tasks.cc"),
                os.path.join(wrap, "ocean_tasks.cc")]
        dirs = [os.path.join(HERE, "shim"), REF, HERE, wrap, os.path.join(root, "include")]
        for name, src in zip(FLW_UNITS, srcs):
            _write_if_changed(os.path.join(FLW_DIR, name), amalgamate(src, dirs, _label))
    units = [os.path.join(FLW_DIR, n) for n in FLW_UNITS]
    if not all(os.path.exists(u) for u in units):
        return None
    extra = os.path.join(HERE, "sw_extra.c")
    out = os.path.join(out_dir, "libref_gb300_L1_T1.so")
    if not (force or _stale(out, units + [extra, os.path.join(HERE, "build.py")])):
        return out
    defs = ["-DMPASO_REF_NVL=1", "-DMPASO_REF_NTR=1", f"-DMPASO_REF_GRAVITY={GRAVITY}"]

    def compile_unit(u):
        obj = os.path.join(out_dir, "gb300_" + os.path.basename(u) + ".o")
        _run(["g++", "-std=c++17", *CFLAGS, *defs, "-w", "-c", u, "-o", obj])
        return obj

    with ThreadPoolExecutor(max_workers=len(units)) as ex:
        objs = list(ex.map(compile_unit, units))
    obj = os.path.join(out_dir, "gb300_sw_extra.o")
    _run(["gcc", "-std=c11", *CFLAGS, f"-I{HERE}", "-c", extra, "-o", obj])
    objs.append(obj)
    _run(["g++", "-shared", "-o", out, *objs, f"-L{lib_dir}", "-lmpaso", f"-Wl,-rpath,{lib_dir}", "-lm"])
    return out


CSTEP_LEVELS = 2  # levels of the complex-step build of the sw tasks


def build_cstep(force=False):
    """oracle/_ref/libref_cstep_L<L>.so: apps/sw/tasks/solve.cc with complex state
    fields (shim MPASO_REF_COMPLEX_STEP) + ref_cstep.cc; None without a checkout."""
    if not ref_available():
        return None
    out_dir = os.path.join(HERE, "_ref")
    os.makedirs(out_dir, exist_ok=True)
    shim = os.path.join(HERE, "shim")
    deps = [os.path.join(dp, f) for dp, _, fs in os.walk(shim) for f in fs]
    deps += [os.path.join(HERE, f) for f in ("ref_cstep.cc", "oracle.h", "build.py")]
    out = os.path.join(out_dir, f"libref_cstep_L{CSTEP_LEVELS}.so")
    if not (force or _stale(out, deps)):
        return out
    defs = [f"-DMPASO_REF_NVL={CSTEP_LEVELS}", "-DMPASO_REF_NTR=1", f"-DMPASO_REF_GRAVITY={GRAVITY}",
            "-DMPASO_REF_COMPLEX_STEP"]
    objs = []
    for path in (os.path.join(REF, "apps/sw/tasks/solve.cc"), os.path.join(HERE, "ref_cstep.cc")):
        obj = os.path.join(out_dir, "cstep_" + os.path.basename(path) + ".o")
        _run(["g++", "-std=c++17", *CFLAGS, *defs, f"-I{shim}", f"-I{REF}", f"-I{HERE}", "-w", "-c", path,
              "-o", obj])
        objs.append(obj)
    _run(["g++", "-shared", "-o", out, *objs, "-lm"])
    return out


if __name__ == "__main__":
    force = "--force" in sys.argv
    print(build_restatement(force))
    print(build_ref(force))
