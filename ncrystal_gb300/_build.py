"""Build steps of the package (no CMake, no setuptools):

* ``build_library()``  -- the CUDA library libncrystal_gb300.so (sm_103a kernels +
  C ABI + table builder), in ncrystal_gb300/_build/.
* ``build_oracle()``   -- the CPU oracle liboracle.so in oracle/_build/ (test
  infrastructure, never loaded by the library).
* ``build_reference()`` -- where the NCrystal sources exist: the reference
  library (oracle/ref.mk), the bundle exporter and the refpin harness, in
  oracle/_ref/.
* ``export_bundles()`` -- material bundles for the workload materials into
  ncrystal_gb300/bundles/ (needs the reference build).

Compiles run in parallel; everything is quick enough to redo on the GPU host.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INC = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
ORACLE = os.path.join(ROOT, "oracle")
ORACLE_BUILD = os.path.join(ORACLE, "_build")
REF_OUT = os.path.join(ORACLE, "_ref")
BUNDLES = os.path.join(PKG, "bundles")
# NCrystal source tree (test oracle and bundle export only): NCGB_REFERENCE_DIR,
# else a checkout named "reference" beside this repository.
REFDIR = os.environ.get("NCGB_REFERENCE_DIR") or os.path.join(os.path.dirname(ROOT), "reference")

LIBNAME = "libncrystal_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nv = shutil.which("nvcc")
    if nv:
        return os.path.dirname(os.path.dirname(os.path.realpath(nv)))
    raise RuntimeError("nvcc not found: the GPU library cannot be built")


def _run(cmd, cwd=None):
    r = subprocess.run(cmd, cwd=cwd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed (%d): %s\n%s" % (r.returncode, " ".join(cmd), r.stdout))
    return r.stdout


def _newer(target, sources):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources)


def _headers():
    hs = [os.path.join(INC, f) for f in os.listdir(INC) if f.endswith(".h")]
    hs += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".hh", ".cuh"))]
    return hs


def library_path():
    return os.path.join(BUILD, LIBNAME)


def oracle_path():
    return os.path.join(ORACLE_BUILD, "liboracle.so")


def build_library(force=False, verbose=False):
    """Compile the CUDA library for sm_103a.  Returns the .so path."""
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(BUILD, exist_ok=True)
    cu = ["ncgb_kernels.cu", "ncgb_noalloc.cu", "ncgb_mlp.cu", "ncgb_mmc.cu", "ncgb_sabderive.cu"]
    # the device table builder shares its arithmetic with the host builder
    # (g++ -ffp-contract=off): no contraction into FMAs there either
    cu_flags = {"ncgb_sabderive.cu": ["-fmad=false"]}
    cc = ["ncgb_capi.cc", "ncgb_tables.cc", "ncgb_bundle.cc", "ncgb_hostapi.cc", "ncgb_proposal.cc",
          "ncgb_mmc.cc"]
    hdrs = _headers()
    jobs = []
    objs = []
    for f in cu:
        src = os.path.join(CSRC, f)
        obj = os.path.join(BUILD, f + ".o")
        objs.append(obj)
        if force or not _newer(obj, [src] + hdrs):
            jobs.append([nvcc] + ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC"]
                        + cu_flags.get(f, []) + ["-I" + INC, "-I" + CSRC, "-c", src, "-o", obj])
    for f in cc:
        src = os.path.join(CSRC, f)
        obj = os.path.join(BUILD, f + ".o")
        objs.append(obj)
        if force or not _newer(obj, [src] + hdrs):
            jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall",
                         "-I" + INC, "-I" + CSRC, "-I" + os.path.join(cuda, "include"),
                         "-c", src, "-o", obj])
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            if o.strip():
                print(o)
    lib = library_path()
    if force or jobs or not os.path.exists(lib):
        # -Bsymbolic: the library's own calls to its exported NCrystal-named
        # symbols bind inside it, even in a process that has NCrystal loaded
        # (the plugin, the on-demand exporter)
        _run([nvcc] + ARCH + ["-shared", "-Xlinker", "-Bsymbolic", "-o", lib] + objs + ["-lcudart", "-ldl"])
    return lib


def build_oracle(force=False):
    """Compile the CPU oracle (test infrastructure)."""
    os.makedirs(ORACLE_BUILD, exist_ok=True)
    srcs = [os.path.join(ORACLE, "ncgb_oracle.c"), os.path.join(ORACLE, "ncgb_oracle_mmc.c")]
    out = oracle_path()
    deps = srcs + [os.path.join(INC, "ncgb_philox.h"), os.path.join(INC, "ncgb_tables.h")]
    if force or not _newer(out, deps):
        _run(["gcc", "-std=gnu99", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-I" + INC,
              "-o", out] + srcs + ["-lm"])
    return out


def reference_available():
    return os.path.exists(os.path.join(REFDIR, "ncrystal_core", "src"))


def build_reference(jobs=None):
    """Build the reference library, the exporter and refpin (where the
    reference sources exist).  Returns False if they do not."""
    if not reference_available():
        return False
    jobs = jobs or os.cpu_count() or 4
    _run(["make", "-s", "-f", os.path.join(ORACLE, "ref.mk"), "-j%d" % jobs,
          "REFDIR=" + REFDIR, "OUT=" + REF_OUT], cwd=ROOT)
    core = os.path.join(REFDIR, "ncrystal_core", "include")
    gen = os.path.join(REF_OUT, "gen")
    bdir = os.path.join(PKG, "bundle")
    exp_src = os.path.join(bdir, "ncgb_export.cc")
    exp_deps = [exp_src, os.path.join(bdir, "ncgb_export.hh")]
    exp_out = os.path.join(REF_OUT, "ncgb_export")
    plug_src = os.path.join(PKG, "plugin", "ncgb_plugin.cc")
    rp_src = os.path.join(ORACLE, "refpin.c")
    rp_out = os.path.join(REF_OUT, "librefpin.so")
    lib = os.path.join(REF_OUT, "libNCrystal.so")
    cxx = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-include", "stdexcept", "-I" + gen, "-I" + core,
           "-I" + bdir]
    link = ["-L" + REF_OUT, "-lNCrystal", "-Wl,-rpath," + REF_OUT]
    cmds = []
    if not _newer(exp_out, exp_deps + [lib]):
        cmds.append(cxx + ["-DNCGB_EXPORT_TOOL", "-o", exp_out, exp_src] + link)
    # the on-demand exporter the library loads for cfg-strings without a
    # bundle, and the NCrystal plugin; both beside the library
    os.makedirs(BUILD, exist_ok=True)
    if not _newer(exporter_path(), exp_deps + [lib]):
        cmds.append(cxx + ["-fPIC", "-shared", "-o", exporter_path(), exp_src] + link)
    if not _newer(plugin_path(), exp_deps + [plug_src, lib]):
        cmds.append(cxx + ["-fPIC", "-shared", "-o", plugin_path(), plug_src, exp_src] + link + ["-ldl"])
    if not _newer(rp_out, [rp_src, lib, os.path.join(INC, "ncgb_philox.h")]):
        cmds.append(["gcc", "-std=c99", "-O2", "-fPIC", "-shared", "-ffp-contract=off",
                     "-I" + INC, "-I" + gen, "-I" + core, "-o", rp_out, rp_src,
                     "-L" + REF_OUT, "-lNCrystal", "-Wl,-rpath," + REF_OUT])
    with ThreadPoolExecutor(max_workers=max(1, len(cmds))) as ex:
        list(ex.map(_run, cmds))
    return True


def exporter_path():
    """libncgb_export.so: NCrystal's material loading, exported as a bundle on
    demand (built where the NCrystal sources are)."""
    return os.path.join(BUILD, "libncgb_export.so")


def plugin_path():
    """The NCrystal plugin libNCrystalPlugin_GB300.so (built where the NCrystal
    sources are)."""
    return os.path.join(BUILD, "libNCrystalPlugin_GB300.so")


def bundle_file_name(cfg):
    """Same canonical form and file name as the C ABI's bundle lookup."""
    s = "".join(c for c in cfg if not c.isspace())
    parts = s.split(";")
    params = sorted(p for p in parts[1:] if p)
    canon = ";".join([parts[0]] + params)
    return "".join(c if (c.isalnum() or c in ".=-_") else "_" for c in canon) + ".ncgb"


def export_bundles(cfgs, outdir=None, with_derived=False, force=False):
    """Run the exporter for each cfg-string.  Returns {cfg: path}."""
    outdir = outdir or BUNDLES
    os.makedirs(outdir, exist_ok=True)
    exp = os.path.join(REF_OUT, "ncgb_export")
    if not os.path.exists(exp):
        raise RuntimeError("bundle exporter not built (needs the NCrystal sources)")
    res = {}
    todo = []
    for cfg in cfgs:
        path = os.path.join(outdir, bundle_file_name(cfg))
        res[cfg] = path
        # re-export when the exporter is newer than the bundle (new records)
        if force or not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(exp):
            cmd = [exp] + (["--with-derived"] if with_derived else []) + [path, cfg]
            todo.append(cmd)
    env = dict(os.environ)
    env["NCRYSTAL_FACTORY_THREADS"] = "1"
    with ThreadPoolExecutor(max_workers=min(8, max(1, len(todo)))) as ex:
        list(ex.map(lambda c: _run(c), todo))
    return res


if __name__ == "__main__":
    print(build_library(force="--force" in sys.argv, verbose=True))
    print(build_oracle(force="--force" in sys.argv))
