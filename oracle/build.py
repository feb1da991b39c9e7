"""Builds the oracle's C restatement and its C++ triangulator (test
infrastructure) into oracle/lib/, and the reference's own C++ modules into
oracle/_ref/ when the reference sources and pybind11 are available."""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "lib", "liboracle.so")
CDT = os.path.join(HERE, "lib", "libcdt3.so")


def build_oracle_c():
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    src = os.path.join(HERE, "limgrad.c")
    if os.path.exists(LIB) and os.path.getmtime(LIB) > os.path.getmtime(src):
        return LIB
    subprocess.run(["gcc", "-O2", "-shared", "-fPIC", "-ffp-contract=off", src, "-o", LIB, "-lm"], check=True)
    return LIB


def build_cdt():
    """the exact-predicate C++ triangulator (oracle/cdt3.cpp); returns None,
    after a note on stderr, when no C++ compiler builds it"""
    src = os.path.join(HERE, "cdt3.cpp")
    if os.path.exists(CDT) and os.path.getmtime(CDT) > os.path.getmtime(src):
        return CDT
    os.makedirs(os.path.dirname(CDT), exist_ok=True)
    cmd = ["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-ffp-contract=off", src, "-o", CDT + ".tmp"]
    try:
        subprocess.run(cmd, check=True, capture_output=True, text=True)
        os.replace(CDT + ".tmp", CDT)
    except (OSError, subprocess.CalledProcessError) as e:
        err = getattr(e, "stderr", "") or str(e)
        print("oracle: the C++ triangulator was not built: " + err.strip()[:500], file=sys.stderr)
        return None
    return CDT


def reference_dir():
    """the reference checkout: $SEISMICMESH_REF, else a directory named
    `reference` beside this repository"""
    return os.environ.get("SEISMICMESH_REF",
                          os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference"))


def build_ref():
    ref = reference_dir()
    if not os.path.isdir(ref):
        return None
    try:
        import pybind11  # noqa: F401
    except ImportError:
        return None
    subprocess.run(["make", "-s", "-C", HERE, f"REF={ref}"], check=True)
    return os.path.join(HERE, "_ref")


def build_all():
    build_oracle_c()
    build_cdt()
    build_ref()


if __name__ == "__main__":
    build_all()
