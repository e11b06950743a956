"""Build recipe for the CPU oracle — TEST INFRASTRUCTURE ONLY.

`build_oracle()` compiles oracle.cpp (the restatement) into oracle/liboracle.so with
-ffp-contract=off so that x86-64 and aarch64 hosts produce identical bits.
`build_ref()` compiles oracle/ref_plgsy_main.cpp against the reference's own
examples/potrf/core_plgsy.h where it lies in a reference checkout (if one is present),
writing only into oracle/_ref/.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))


def _find_reference():
    """The reference checkout: $TTG_REFERENCE_ROOT, else a `reference` directory beside the
    repository's own directory; None when neither holds examples/potrf."""
    env = os.environ.get("TTG_REFERENCE_ROOT")
    cands = [env] if env else [os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")]
    for c in cands:
        if c and os.path.isdir(os.path.join(c, "examples", "potrf")):
            return c
    return None


REF_ROOT = _find_reference() or ""


def _newer(out, srcs):
    return os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(s) for s in srcs)


def build_oracle(force=False):
    src = os.path.join(HERE, "oracle.cpp")
    hdr = os.path.join(HERE, "oracle.h")
    out = os.path.join(HERE, "liboracle.so")
    if not force and _newer(out, [src, hdr]):
        return out
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-pthread",
           src, "-o", out + ".tmp", "-ldl"]
    subprocess.check_call(cmd)
    os.replace(out + ".tmp", out)
    return out


def build_ref(force=False):
    """Returns the path of the reference generator binary, or None without a reference checkout."""
    hdr = os.path.join(REF_ROOT, "examples", "potrf", "core_plgsy.h")
    if not REF_ROOT or not os.path.exists(hdr):
        return None
    src = os.path.join(HERE, "ref_plgsy_main.cpp")
    outdir = os.path.join(HERE, "_ref")
    os.makedirs(outdir, exist_ok=True)
    out = os.path.join(outdir, "ref_plgsy")
    if not force and _newer(out, [src, hdr]):
        return out
    cmd = ["g++", "-std=c++17", "-O2", "-I", os.path.dirname(hdr), src, "-o", out]
    subprocess.check_call(cmd)
    return out


def _cuda_inc():
    for d in ("/usr/local/cuda/include",):
        if os.path.isdir(d):
            return d
    return "/usr/local/cuda/include"


def build_ref_flowgraph(force=False):
    """Compiles the reference's own potrf flowgraph (examples/potrf/potrf.h, plgsy.h, result.h,
    pmw.h, ../matrixtile.h) and its unmodified driver testing_dpotrf.cc against this project's
    ttg.h, with the PaRSEC/LAPACK stand-ins of oracle/ref_shim and the oracle's tile kernels.
    Returns (ref_potrf, testing_dpotrf) paths, or None without a reference checkout."""
    potrf_dir = os.path.join(REF_ROOT, "examples", "potrf")
    if not REF_ROOT or not os.path.exists(os.path.join(potrf_dir, "potrf.h")):
        return None
    root = os.path.dirname(HERE)
    outdir = os.path.join(HERE, "_ref")
    os.makedirs(outdir, exist_ok=True)
    common = ["g++", "-std=c++20", "-O2", "-ffp-contract=off", "-pthread",
              "-I", os.path.join(HERE, "ref_shim"), "-I", HERE, "-I", os.path.join(root, "include"),
              "-I", potrf_dir, "-I", os.path.dirname(potrf_dir), "-I", _cuda_inc()]
    libs = ["-L/usr/local/cuda/lib64", "-lcudart", "-ldl"]
    deps = [os.path.join(HERE, f) for f in ("oracle.cpp", "oracle.h", "ref_potrf_main.cpp", "ref_shim/parsec.h",
                                            "ref_shim/lapack.hh")]
    deps += [os.path.join(root, "include", "ttg", f) for f in ("tt.h", "runtime.h", "buffer.h", "device/task.h")]
    outs = []
    for name, src in (("ref_potrf", os.path.join(HERE, "ref_potrf_main.cpp")),
                      ("testing_dpotrf", os.path.join(potrf_dir, "testing_dpotrf.cc"))):
        out = os.path.join(outdir, name)
        if force or not _newer(out, deps + [src]):
            subprocess.check_call(common + [src, os.path.join(HERE, "oracle.cpp"), "-o", out] + libs)
        outs.append(out)
    return tuple(outs)


if __name__ == "__main__":
    print(build_oracle(force=True))
    print(build_ref(force=True))
    print(build_ref_flowgraph(force=True))
