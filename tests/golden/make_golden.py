"""Generate the golden fixtures in this directory from the REFERENCE ITSELF.

Runs only where the reference checkout is present: it builds the reference's
CPU path from its own sources (oracle/ref/Makefile, protobuf shim) and runs
its ``test_compress_cpu`` and the ``ref_dump`` glue on seeded inputs.  The
outputs committed here pin the oracle and the GPU library on machines without
the reference.

    python tests/golden/make_golden.py [/path/to/reference]

Writes, per case: ``<case>.in.cube`` (input), ``<case>.<p>.cube`` (reference
compressed output), ``<case>.<p>.d.cube`` (reference decompression of it),
``<case>.<p>.coeffs.f32`` (reference transform output, rotated Z-X-Y order),
``<case>.<o>.opt.txt`` (the table the reference's -opt sweep prints),
``<case>.<p>.err.txt`` (the error line the reference's -err prints; float
inputs also from a copy ``<case>.max1.in.cube`` whose maximum_value is 1) and
``manifest.json`` (flags, sizes, threshold statistics, hashes).  ``--err``
regenerates only the -err fixtures.
"""
import hashlib
import json
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import build_oracle  # noqa: E402
from wavelets_gb300 import cubefile, synth  # noqa: E402

PARAMS = {
    "p1": ["-steps", "-1", "-thresh", "0.5", "-qalg", "log", "-qcount", "256"],
    "p2": ["-steps", "3,3,3", "-thresh", "0.95", "-qalg", "uniform", "-qcount", "1024"],
    "p3": ["-wave", "haar", "-steps", "2,2,2", "-thresh", "0.9", "-qalg", "lloyd", "-qcount", "256"],
    "p4": ["-steps", "2,1", "-thresh", "0.7", "-qalg", "log", "-qcount", "255", "-noz"],
    "p5": ["-wave", "haar", "-thresh", "0.8", "-qalg", "uniform", "-qcount", "7"],
    "p6": ["-steps", "0,0,0", "-thresh", "0.6", "-qalg", "log", "-qcount", "64"],
    "p7": ["-steps", "4,4,4", "-thresh", "0.9", "-qalg", "lloyd", "-qcount", "255"],
    # -2d: a 2-D transform of every z layer (test_compress_common.cc:519-541)
    "p8": ["-2d", "-steps", "-1", "-thresh", "0.8", "-qalg", "log", "-qcount", "256"],
    "p9": ["-2d", "-wave", "haar", "-steps", "3,2", "-thresh", "0.9", "-qalg", "uniform",
           "-qcount", "512"],
    # x steps 0 mean the maximum in 2-D mode; z steps still pad the layers
    "p10": ["-2d", "-steps", "0,2,3", "-thresh", "0.7", "-qalg", "log", "-qcount", "255"],
}

# -opt sweeps (optimizeParameters -> plotAll): the printed table is the fixture
OPT = {"o1": ["-opt"], "o2": ["-opt", "-2d", "-steps", "3,2"],
       "o3": ["-opt", "-noz", "-wave", "haar", "-steps", "2,2,2"]}
OPT_CASES = {"uint8_1x64x64": ["o1", "o2", "o3"], "uint8_2x33x17": ["o1"]}

# extra -2d parameter sets per case
PLANS_2D = {"uint8_1x64x64": ["p8", "p10"], "float32_12x20x24": ["p9"],
            "uint8_5x7x9": ["p8", "p10"], "uint16_16x16x16": ["p8", "p9"]}

# (case name, array, parameter sets)
def cases():
    out = []
    small = synth.small_cases()
    plans = [["p1", "p2", "p3"], ["p1", "p4", "p7"], ["p2", "p5", "p6"],
             ["p1", "p5"], ["p2", "p3", "p7"], ["p1", "p4"], ["p3", "p6"],
             ["p1", "p2", "p4"]]
    for (name, arr), plan in zip(small, plans):
        out.append((name, arr, plan + PLANS_2D.get(name, [])))
    rng = np.random.default_rng(11)
    img = synth.scaled_blob_cubelet(rng, (1, 256, 256), np.uint8)
    out.append(("uint8_1x256x256", img, ["p1", "p4"]))
    # all-zero and constant cubes: threshold 0 -> 1e-16, single Huffman symbol
    out.append(("float32_4x4x4_zero", np.zeros((4, 4, 4), np.float32), ["p1"]))
    out.append(("uint8_1x8x8_const", np.full((1, 8, 8), 7, np.uint8), ["p2"]))
    return out


def sha(path):
    with open(path, "rb") as f:
        return hashlib.sha256(f.read()).hexdigest()


def kat_cdf97(ref_dump, tmp):
    """cdf97 one step on the vector of dwt_cpu.cc:657 (x axis only)."""
    v = np.array([7, 2, 3, 4, 5, 3, 1, 5, 7, 1, 9, 2, 4, 8, 2, 6], np.float32)
    path = os.path.join(tmp, "kat.cube")
    cubefile.write_file(path, [cubefile.from_array(v.reshape(1, 1, 16))])
    d = os.path.join(tmp, "katdump")
    os.makedirs(d, exist_ok=True)
    subprocess.check_call([ref_dump, "-steps", "1,0,0", path,
                           os.path.join(tmp, "kat.out.cube"), d])
    return np.fromfile(os.path.join(d, "coeffs.f32"), np.float32)


# -err fixtures: the reference's printed error line for these (case, params)
# pairs; float32 inputs also as a copy whose maximum_value is set to 1 (the
# reference computes nothing for float input without one)
ERR_CASES = [("uint8_1x64x64", "p1"), ("uint8_1x64x64", "p3"), ("uint8_2x33x17", "p3"),
             ("uint8_5x7x9", "p1"), ("uint8_1x256x256", "p4"), ("uint16_16x16x16", "p2"),
             ("uint16_16x16x16", "p7"), ("float32_8x16x32", "p1"), ("float32_8x16x32", "p4"),
             ("float32_12x20x24", "p2"), ("float32_3x2x5", "p5")]


def make_err(cli, manifest):
    """Run the reference with -err on ERR_CASES; write <case>.<p>.err.txt
    (its stdout) and manifest["err"]."""
    out = []
    with tempfile.TemporaryDirectory() as tmp:
        for name, p in ERR_CASES:
            inputs = [(name + ".in.cube", "")]
            if name.startswith("float32"):
                c = cubefile.read_file(os.path.join(HERE, name + ".in.cube"))[0]
                m1 = name + ".max1.in.cube"
                cubefile.write_file(os.path.join(HERE, m1),
                                    [cubefile.from_array(c.array(), maximum_value=1)])
                inputs.append((m1, ".max1"))
            for inp, tag in inputs:
                txt = f"{name}{tag}.{p}.err.txt"
                r = subprocess.run([cli, "-q", "-err", *PARAMS[p], os.path.join(HERE, inp),
                                    os.path.join(tmp, "x.cube")],
                                   capture_output=True, text=True, check=True)
                line = [ln for ln in r.stdout.splitlines() if ln.startswith("Mean squared")]
                with open(os.path.join(HERE, txt), "w") as f:
                    f.write("\n".join(line) + "\n")
                out.append({"case": name, "params": p, "input": inp, "err": txt})
    manifest["err"] = out


def main():
    if len(sys.argv) > 1 and sys.argv[1] == "--err":
        # only the -err fixtures, added to the existing manifest
        ref = sys.argv[2] if len(sys.argv) > 2 else build_oracle.reference_dir()
        if not ref or not os.path.isdir(ref):
            sys.exit("reference checkout not found: pass its path or set WL_REFERENCE_DIR")
        build_oracle.build_reference(ref)
        mpath = os.path.join(HERE, "manifest.json")
        manifest = json.load(open(mpath))
        make_err(os.path.join(ROOT, "oracle", "_ref", "test_compress_cpu"), manifest)
        with open(mpath, "w") as f:
            json.dump(manifest, f, indent=1)
        print("wrote", len(manifest["err"]), "-err fixtures")
        return
    ref = sys.argv[1] if len(sys.argv) > 1 else build_oracle.reference_dir()
    if not ref or not os.path.isdir(ref):
        sys.exit("reference checkout not found: pass its path or set WL_REFERENCE_DIR")
    build_oracle.build_reference(ref)
    cli = os.path.join(ROOT, "oracle", "_ref", "test_compress_cpu")
    dump = os.path.join(ROOT, "oracle", "_ref", "ref_dump")
    manifest = {"generator": "tests/golden/make_golden.py",
                "params": PARAMS, "cases": []}
    with tempfile.TemporaryDirectory() as tmp:
        kat = kat_cdf97(dump, tmp)
        manifest["kat_cdf97_1step"] = {
            "input": [7, 2, 3, 4, 5, 3, 1, 5, 7, 1, 9, 2, 4, 8, 2, 6],
            "output_hex": [float(x).hex() for x in kat],
            # printed in the reference's comment dwt_cpu.cc:680
            "published": [7.00224, 3.52709, 6.82547, 2.87912, 7.34827, 7.39307,
                          6.14146, 6.57857, 2.33178, -0.122068, -0.136087,
                          -1.33848, 5.86312, 3.64358, -4.18374, -2.92383]}
        for name, arr, plan in cases():
            inp = os.path.join(HERE, name + ".in.cube")
            cubefile.write_file(inp, [cubefile.from_array(arr)])
            for p in plan:
                out = os.path.join(HERE, f"{name}.{p}.cube")
                dec = os.path.join(HERE, f"{name}.{p}.d.cube")
                subprocess.check_call([cli, "-q", *PARAMS[p], inp, out])
                subprocess.check_call([cli, "-q", "-d", out, dec])
                d = os.path.join(tmp, name + p)
                os.makedirs(d)
                subprocess.check_call([dump, *PARAMS[p], inp,
                                       os.path.join(tmp, "x.cube"), d])
                shutil.copy(os.path.join(d, "coeffs.f32"),
                            os.path.join(HERE, f"{name}.{p}.coeffs.f32"))
                stats = {}
                with open(os.path.join(d, "stats.txt")) as f:
                    lines = f.read().split("\n")
                for ln in lines[:8]:
                    parts = ln.split()
                    if parts:
                        stats[parts[0]] = parts[1:]
                manifest["cases"].append({
                    "case": name, "params": p, "shape_zyx": list(arr.shape),
                    "dtype": str(arr.dtype), "input": os.path.basename(inp),
                    "output": os.path.basename(out),
                    "decompressed": os.path.basename(dec),
                    "coeffs": f"{name}.{p}.coeffs.f32",
                    "stats": stats,
                    "sha256": {"output": sha(out), "decompressed": sha(dec)}})
        manifest["opt"] = {"params": OPT, "cases": []}
        for name, plan in OPT_CASES.items():
            inp = os.path.join(HERE, name + ".in.cube")
            for o in plan:
                txt = os.path.join(HERE, f"{name}.{o}.opt.txt")
                r = subprocess.run([cli, "-q", *OPT[o], inp, os.path.join(tmp, "none.cube")],
                                   capture_output=True, text=True, check=True)
                with open(txt, "w") as f:
                    f.write(r.stdout)
                manifest["opt"]["cases"].append({"case": name, "params": o,
                                                 "input": os.path.basename(inp),
                                                 "table": os.path.basename(txt)})
        make_err(cli, manifest)
    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1)
    print("wrote", len(manifest["cases"]), "cases")


if __name__ == "__main__":
    main()
