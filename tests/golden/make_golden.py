"""Generates the committed golden fixtures in tests/golden/.

  pcg64dxsm_numpy.json  NumPy's PCG64DXSM (an independent implementation of the
                        generator rand_pcg's Lcg128CmDxsm64 implements) with
                        the state set directly: raw outputs and advance().
  ziggurat_ref.json     SHA-256 of the reference's ziggurat table doubles
                        (src/dist/ziggurat_tables.rs), so the table pin
                        travels without copying the table.

Run from the repository root in a container where the reference tree is
mounted (only the ziggurat part needs it):
    python tests/golden/make_golden.py [/path/to/reference]
"""
from __future__ import annotations

import hashlib
import json
import os
import re
import struct
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def pcg_cases():
    rng = np.random.default_rng(20261203)
    cases = []
    seeds = [(0, 1), (42, 0), (2**64 + 7, 3), (2**127 + 12345, 99)]
    for extra in range(4):
        seeds.append((int.from_bytes(rng.bytes(16), "little"), int.from_bytes(rng.bytes(16), "little")))
    for state, stream in seeds:
        inc = ((stream << 1) | 1) & (2**128 - 1)
        bg = np.random.PCG64DXSM()
        st = bg.state
        st["state"] = {"state": state, "inc": inc}
        bg.state = st
        outs = [int(x) for x in bg.random_raw(16)]
        adv = []
        for delta in (1, 1000, 2**40 + 3, 2**100 + 5):
            bg.state = st
            bg.advance(delta)
            adv.append({"delta": str(delta), "state": str(bg.state["state"]["state"]),
                        "next": str(int(bg.random_raw(1)[0]))})
        cases.append({"state": str(state), "inc": str(inc), "outputs": [str(o) for o in outs], "advance": adv})
    return cases


def table_hash(ref_root: str):
    src = open(os.path.join(ref_root, "src/dist/ziggurat_tables.rs")).read()

    def arr(name):
        body = src.split(f"pub const {name}: [f64; 257] = [")[1].split("];")[0]
        return [float(v) for v in re.findall(r"([-0-9.e+]+),", body)]

    x, y = arr("ZIGGURAT_X"), arr("ZIGGURAT_Y")
    r = float(re.search(r"ZIGGURAT_R: f64 = ([0-9.e+-]+);", src).group(1))
    pack = lambda v: struct.pack("<%dd" % len(v), *v)
    return {"n_x": len(x), "n_y": len(y), "r": r.hex(),
            "sha256_x": hashlib.sha256(pack(x)).hexdigest(), "sha256_y": hashlib.sha256(pack(y)).hexdigest()}


def main():
    with open(os.path.join(HERE, "pcg64dxsm_numpy.json"), "w") as f:
        json.dump({"generator": "numpy.random.PCG64DXSM", "numpy": np.__version__, "cases": pcg_cases()}, f,
                  indent=1)
    # the reference checkout: first argument, else STOCHA_REFERENCE_ROOT
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("STOCHA_REFERENCE_ROOT", "")
    if ref and os.path.exists(os.path.join(ref, "src/dist/ziggurat_tables.rs")):
        with open(os.path.join(HERE, "ziggurat_ref.json"), "w") as f:
            json.dump(table_hash(ref), f, indent=1)


if __name__ == "__main__":
    main()
