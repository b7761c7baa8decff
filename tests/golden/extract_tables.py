"""Extract the reference's Marching Cubes lookup tables into tests/golden/ref_tables.json.

Runs only where the reference checkout is present: its path is the REF environment variable
(required).  The JSON is a golden fixture: tests compare the tables this library
generates (tmc_gb300/csrc/mc_tables.h) against it, and tmc_gb300/csrc/gen_tables.py packs the
two tables that are arbitrary data (the contour start edges of cpp_dmc/LookupTables.h r_pattern
and the triangle list mc/MarchingCubes.h t_pattern) from it.

Sources read:
  mc/MarchingCubes.h        e_pattern[256], t_pattern[4096], t_ambig[256]
  cpp_dmc/LookupTables.h    r_pattern[4352], t_ambig[256]
"""
import json
import os
import re
import sys

REF = os.environ.get("REF", "")
HERE = os.path.dirname(os.path.abspath(__file__))


def grab(path: str, name: str):
    lines = open(path).read().split("\n")
    for i, line in enumerate(lines):
        s = line.strip()
        if s.startswith("//"):
            continue
        if re.search(r"\b" + name + r"\b\s*(\[|=)", s) and "const" in s:
            buf = []
            for l2 in lines[i:]:
                buf.append(l2.split("//")[0])
                if "};" in l2:
                    break
            txt = " ".join(buf)
            body = txt[txt.index("{") + 1:]
            body = body[: body.rindex("}")].replace("{", " ").replace("}", " ")
            return [int(x, 0) for x in re.findall(r"-?0x[0-9a-fA-F]+|-?\d+", body)]
    raise KeyError(name)


def main():
    if not os.path.isdir(REF):
        print("reference checkout not found at", REF, file=sys.stderr)
        return 1
    t = {
        "mc_e_pattern": grab(f"{REF}/mc/MarchingCubes.h", "e_pattern"),
        "mc_t_pattern": grab(f"{REF}/mc/MarchingCubes.h", "t_pattern"),
        "mc_t_ambig": grab(f"{REF}/mc/MarchingCubes.h", "t_ambig"),
        "dmc_r_pattern": grab(f"{REF}/cpp_dmc/LookupTables.h", "r_pattern"),
        "dmc_t_ambig": grab(f"{REF}/cpp_dmc/LookupTables.h", "t_ambig"),
    }
    assert len(t["mc_e_pattern"]) == 256 and len(t["mc_t_pattern"]) == 4096
    assert len(t["dmc_r_pattern"]) == 4352 and len(t["mc_t_ambig"]) == 256
    with open(os.path.join(HERE, "ref_tables.json"), "w") as f:
        json.dump(t, f, separators=(",", ":"))
    return 0


if __name__ == "__main__":
    sys.exit(main())
