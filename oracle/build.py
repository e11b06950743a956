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
REF_ROOT = os.environ.get("TTG_REFERENCE_ROOT", "/root/reference")


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
    if not os.path.exists(hdr):
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


if __name__ == "__main__":
    print(build_oracle(force=True))
    print(build_ref(force=True))
