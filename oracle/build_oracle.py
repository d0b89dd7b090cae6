"""Build the test oracle (test infrastructure, never shipped).

* ``oracle/_build/liboracle.so`` and ``oracle/_build/oracle_cli``: the CPU
  restatement of the reference path (oracle/port), built on every machine.
* ``oracle/_ref/``: the reference's own CPU path compiled from its sources with
  the protobuf shim (oracle/ref/Makefile), built only where the reference
  checkout is present (pass its location as ``ref_dir``).
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
FLAGS = ["-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-w",
         "-I" + os.path.join(HERE, "shim"), "-I" + os.path.join(HERE, "port")]


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build_port(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "port", "wl_port.cpp")
    deps = [src, os.path.join(HERE, "port", "wl_port.h"),
            os.path.join(HERE, "shim", "wavelet_compress.pb.h")]
    lib = os.path.join(BUILD, "liboracle.so")
    cli = os.path.join(BUILD, "oracle_cli")
    if _stale(lib, deps):
        subprocess.check_call(["g++", *FLAGS, "-shared", src, "-o", lib])
    cli_src = os.path.join(HERE, "port", "port_cli.cpp")
    if _stale(cli, deps + [cli_src]):
        subprocess.check_call(["g++", *FLAGS, cli_src, src, "-o", cli])
    return lib, cli


def reference_dir():
    """The reference checkout: $WL_REFERENCE_DIR, else a directory named
    `reference` beside this repository (None when neither exists; the GPU
    box has no checkout, and nothing there needs one)."""
    d = os.environ.get("WL_REFERENCE_DIR") or os.path.join(
        os.path.dirname(os.path.dirname(HERE)), "reference")
    return d if os.path.isdir(d) else None


def build_reference(ref_dir):
    """Compile the reference CPU path (only where its sources exist)."""
    if not ref_dir or not os.path.isdir(ref_dir):
        return None
    subprocess.check_call(["make", "-s", "-C", os.path.join(HERE, "ref"),
                           "REF=" + ref_dir, "-j8"])
    return os.path.join(HERE, "_ref", "test_compress_cpu")


if __name__ == "__main__":
    print(build_port())
