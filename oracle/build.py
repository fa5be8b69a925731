"""Build recipes for the CPU oracles. TEST INFRASTRUCTURE ONLY.

``build_port()`` compiles the C restatement (oracle/port/eif_port.c) into
oracle/port/libeifport.so on any machine. ``build_ref()`` compiles the
reference's own sources into oracle/_ref/ with oracle/ref/Makefile, which is
possible only where the reference sources exist: the checkout named by
EIF_REFERENCE_DIR, else a checkout called ``reference`` beside this repository.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
PORT_SO = os.path.join(HERE, "port", "libeifport.so")
REFERENCE_DIR = os.environ.get("EIF_REFERENCE_DIR") or os.path.join(os.path.dirname(ROOT), "reference")


def build_port(force=False):
    srcs = [os.path.join(HERE, "port", "eif_port.c"), os.path.join(HERE, "ref", "shim", "fftw_shim.c")]
    deps = srcs + [os.path.join(ROOT, "include", "eif.h"), os.path.join(HERE, "ref", "shim", "fftw3.h")]
    if not force and os.path.exists(PORT_SO):
        t = os.path.getmtime(PORT_SO)
        if all(os.path.getmtime(d) <= t for d in deps):
            return PORT_SO
    cmd = ["gcc", "-O2", "-std=c99", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
           "-D_POSIX_C_SOURCE=200809L", "-I" + os.path.join(ROOT, "include"),
           "-I" + os.path.join(HERE, "ref", "shim")] + srcs + ["-lm", "-o", PORT_SO + ".tmp"]
    subprocess.check_call(cmd)
    os.replace(PORT_SO + ".tmp", PORT_SO)
    return PORT_SO


def build_ref():
    """Build oracle/_ref/ from the reference sources; returns False if they are absent."""
    if not os.path.isdir(os.path.join(REFERENCE_DIR, "src")):
        return False
    subprocess.check_call(["make", "-s", "-C", os.path.join(HERE, "ref"), "REF=" + REFERENCE_DIR, "all"])
    return True


if __name__ == "__main__":
    print(build_port(force=True))
    print("reference build:", build_ref())
