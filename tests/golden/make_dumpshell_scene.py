"""Regenerate dumpshell_scene.json: the scene the reference's DumpShell test rebuilds from
b2World.Dump-style text (examples/demo/tests/dumpshell.d, a dumped scene of Box2D issue 304),
read as text through dbox_gb300.dump.parse and stored as plain numbers.

Run from the repository root:  python tests/golden/make_dumpshell_scene.py <dbox checkout>/examples/demo/tests/dumpshell.d
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))

from dbox_gb300 import dump  # noqa: E402


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: make_dumpshell_scene.py <dbox checkout>/examples/demo/tests/dumpshell.d")
    src = sys.argv[1]
    p = dump.parse(open(src).read())
    out = {"source": "examples/demo/tests/dumpshell.d (dbox)", "gravity": list(p["gravity"]),
           "bodies": [{k: (v.tolist() if hasattr(v, "tolist") else v) for k, v in zip(b.dtype.names, b.tolist())}
                      for b in p["bodies"]],
           "fixtures": []}
    for op in p["fixtures"]:
        assert op[0] == "fixture"
        _, body, sd, fd = op
        out["fixtures"].append({"body": body, "kind": int(sd["kind"]), "count": int(sd["count"]),
                                "vertices": sd["vertices"][:int(sd["count"])].tolist(),
                                "friction": float(fd["friction"]), "restitution": float(fd["restitution"]),
                                "density": float(fd["density"]), "is_sensor": int(fd["is_sensor"]),
                                "category_bits": int(fd["category_bits"]), "mask_bits": int(fd["mask_bits"]),
                                "group_index": int(fd["group_index"])})
    with open(os.path.join(HERE, "dumpshell_scene.json"), "w") as f:
        json.dump(out, f, indent=1)
        f.write("\n")


if __name__ == "__main__":
    main()
