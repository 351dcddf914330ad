"""Regenerate the golden fixtures under tests/golden/ (run in a container that
holds a checkout of the reference; the fixtures are committed so that nothing
at test time needs the reference).

1. philox_golden.json: the CoreRow and KeyRow tables of the reference's
   tests/random/golden_random.h (exact Philox bits, uniforms and keys, and the
   tolerance-tier normals), parsed from the header text.
2. ref_cases.npz: inputs and outputs of the reference headers themselves,
   compiled in AETHER_CPP_MODE (oracle/Makefile target `ref`) and run by
   oracle/ref_driver.cpp on seeded inputs from the reference's own Generator.

usage: python tests/golden/make_golden.py [--ref /path/to/reference]
"""

import argparse
import json
import os
import re
import struct
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))


def parse_golden_random(path):
    text = open(path).read()
    core, keys = [], []
    row = re.compile(r"\{\s*([^{}]*?)\s*\},")
    core_block = text.split("kCoreRows[] = {", 1)[1].split("};", 1)[0]
    key_block = text.split("kKeyRows[] = {", 1)[1].split("};", 1)[0]

    def num(tok):
        tok = tok.strip()
        tok = re.sub(r"(ULL|ull|u|U)$", "", tok)
        if tok.startswith("0x") or tok.startswith("0X"):
            return int(tok, 16)
        return int(tok)

    for m in row.finditer(core_block):
        f = [t.strip() for t in m.group(1).split(",")]
        core.append({
            "seed": num(f[0]), "global": num(f[1]), "counter": num(f[2]),
            "bits64": num(f[3]), "uniform_double_bits": num(f[4]), "uniform_float_bits": num(f[5]),
            "normal_double": float(f[6]), "normal_float": float(f[7].rstrip("f")),
        })
    for m in row.finditer(key_block):
        f = [t.strip() for t in m.group(1).split(",")]
        keys.append({"seed": num(f[0]), "stream_id": num(f[1]), "substream_k": num(f[2]),
                     "key": num(f[3]), "substream_key": num(f[4])})
    tol_d = float(re.search(r"kNormalDoubleTol = ([0-9.eE+-]+);", text).group(1))
    tol_f = float(re.search(r"kNormalFloatTol = ([0-9.eE+-]+)f;", text).group(1))
    count = int(re.search(r"kCoreRowCount = (\d+);", text).group(1))
    kcount = int(re.search(r"kKeyRowCount = (\d+);", text).group(1))
    assert len(core) == count and len(keys) == kcount, (len(core), len(keys))
    return {"source": "tests/random/golden_random.h", "core": core, "keys": keys,
            "normal_double_tol": tol_d, "normal_float_tol": tol_f}


def run_reference(ref):
    subprocess.check_call(["make", "-s", "-C", os.path.join(REPO, "oracle"), "ref", "REF=" + ref])
    exe = os.path.join(REPO, "oracle", "_ref", "aether_ref")
    with tempfile.TemporaryDirectory() as d:
        manifest = json.loads(subprocess.check_output([exe, d]))
        arrays = {}
        for m in manifest:
            dt = {"f64": np.float64, "f32": np.float32, "i32": np.int32, "i64": np.int64}[m["dtype"]]
            a = np.fromfile(os.path.join(d, m["name"] + ".bin"), dtype=dt)
            arrays[m["name"]] = a.reshape(m["comps"], m["n"])
    return arrays


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("AETHER_REFERENCE_DIR"),
                    help="checkout of the reference (default: $AETHER_REFERENCE_DIR)")
    args = ap.parse_args()
    if not args.ref:
        ap.error("name the reference checkout with --ref or AETHER_REFERENCE_DIR")
    g = parse_golden_random(os.path.join(args.ref, "tests", "random", "golden_random.h"))
    with open(os.path.join(HERE, "philox_golden.json"), "w") as f:
        json.dump(g, f, indent=0)
    arrays = run_reference(args.ref)
    np.savez_compressed(os.path.join(HERE, "ref_cases.npz"), **arrays)
    print("rows:", len(g["core"]), "keys:", len(g["keys"]), "arrays:", len(arrays))


if __name__ == "__main__":
    main()
