"""Build recipe for the CPU oracle (test infrastructure only).

build_port()      -> oracle/_build/liboracle.so   (the C restatement)
build_reference() -> oracle/_ref/libotfem_ref.so  (unmodified reference headers
                     behind the same C interface; only where the reference
                     tree is present, i.e. not on machines without it)

Both use the pinned parity flags -O2 -ffp-contract=off: no FMA contraction,
so the FP64 operation sequence is exactly the one written in the sources on
x86-64 and on aarch64 alike.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
# The OpenTissue source tree the reference build reads (in place, never
# copied): the environment variable OTFEM_REFERENCE_ROOT, else the recipe's
# default location DEFAULT_REFERENCE_ROOT.  Where neither holds the tree,
# build_reference() builds nothing and the reference-backed checks skip.
DEFAULT_REFERENCE_ROOT = "/root/reference"
REFERENCE_ROOT = os.environ.get("OTFEM_REFERENCE_ROOT", DEFAULT_REFERENCE_ROOT)


def _newer(out, srcs):
    return os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(s) for s in srcs)


def build_port(force=False):
    out_dir = os.path.join(HERE, "_build")
    os.makedirs(out_dir, exist_ok=True)
    out = os.path.join(out_dir, "liboracle.so")
    srcs = [os.path.join(HERE, "otfem_oracle.c"), os.path.join(HERE, "otfem_oracle.h")]
    if force or not _newer(out, srcs):
        cc = os.environ.get("CC", "gcc")
        subprocess.check_call([cc, "-std=c99", "-O2", "-ffp-contract=off", "-fPIC", "-shared",
                               srcs[0], "-o", out, "-lm"])
    return out


def build_reference(force=False):
    """Returns the library path, or None when the reference tree is absent."""
    if not os.path.exists(os.path.join(REFERENCE_ROOT, "OpenTissue", "dynamics", "fem", "fem.h")):
        return None
    out = os.path.join(HERE, "_ref", "libotfem_ref.so")
    srcs = [os.path.join(HERE, "ref", "ref_capi.cpp"), os.path.join(HERE, "ref", "ref_coupling.cpp"),
            os.path.join(HERE, "ref", "build_ref.sh"), os.path.join(HERE, "otfem_oracle.h")]
    if force or not _newer(out, srcs):
        subprocess.check_call(["bash", os.path.join(HERE, "ref", "build_ref.sh"), REFERENCE_ROOT])
    return out


if __name__ == "__main__":
    print(build_port(force=True))
    print(build_reference(force=True))
