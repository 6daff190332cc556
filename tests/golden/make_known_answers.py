"""Extract the reference's operator unit-test vectors into known_answers.json.

Reads the reference's C++ test sources as text (it is never compiled or run
here): for every TEST(Operator, <Name>) block of HashJoin and Mintersect it
records, in order, the input schemas, the std::vector literals, the shapes of
the matrices the test builds (Dense*Matrix(rows, cols)), the operator
constructor arguments and every asserted value (EXPECT_EQ).

    python tests/golden/make_known_answers.py <reference checkout>

The reference checkout is a required argument: the script has no default
location for it.
"""
import json
import re
import sys
from pathlib import Path

FILES = ["src/objects/operator/join.cpp", "src/objects/operator/mintersect.cpp"]
TEST_RE = re.compile(r"^TEST\(Operator,\s*(\w+)\)\s*\{", re.M)
VEC_RE = re.compile(r"std::vector<(\w+)>\s+(\w+)\s*=\s*\{([^}]*)\};")
SCHEMA_RE = re.compile(r"columns\s*=\s*\{(\{\"\w+\",\s*Type::\w+\}(?:,\s*\{\"\w+\",\s*Type::\w+\})*)\}")
COL_RE = re.compile(r"\{\"(\w+)\",\s*Type::(\w+)\}")
MAT_RE = re.compile(r"make_shared<(Dense\w*Matrix)>\((\d+),\s*(\d+)\)")
OP_RE = re.compile(r"new (HashJoin|Mintersect)\(([^)]*)\)")
EXPECT_RE = re.compile(r"EXPECT_EQ\((.*),\s*(\d+)\);")


def blocks(text):
    starts = [(m.group(1), m.end()) for m in TEST_RE.finditer(text)]
    for i, (name, s) in enumerate(starts):
        e = starts[i + 1][1] if i + 1 < len(starts) else len(text)
        yield name, text[s:e], text[:s].count("\n") + 1


SET_RE = re.compile(r"mat->set\((\w+)\[i\],\s*k_map\.at\((\w+)\[i\]\)")


def dependency(seg):
    """One `op->addDependency(...)` block: its schema, table kind, vectors and,
    for a matrix, its shape and how rows and columns are filled."""
    dep = {"schema": [[c, t] for c, t in COL_RE.findall(SCHEMA_RE.search(seg).group(1))],
           "kind": "ColMain" if "ColMainMatrixTable" in seg else "Flat",
           "vectors": {n: [int(x) for x in v.replace(" ", "").split(",") if x]
                       for t, n, v in VEC_RE.findall(seg)}}
    m = MAT_RE.search(seg)
    if m:
        dep["shape"] = [int(m.group(2)), int(m.group(3))]
        st = SET_RE.search(seg)
        dep["set"] = {"row": st.group(1), "col_key": st.group(2)}  # set(row[i], k_map[col_key[i]])
    return dep


def main(ref_root):
    out = {}
    for f in FILES:
        text = (Path(ref_root) / f).read_text()
        for name, body, line in blocks(text):
            op = OP_RE.search(body)
            if not op:
                continue
            segs = body.split("op->addDependency(")[:-1]
            out[name] = {
                "source": f"{f}:{line}",
                "operator": op.group(1),
                "args": [a.strip().strip('"') for a in op.group(2).split(",")],
                "deps": [dependency(sg) for sg in segs],
                "expect": [[lhs.strip(), int(v)] for lhs, v in EXPECT_RE.findall(body)],
            }
    dst = Path(__file__).with_name("known_answers.json")
    dst.write_text(json.dumps(out, indent=1) + "\n")
    print(f"{len(out)} tests -> {dst}")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_known_answers.py <reference checkout>")
    main(sys.argv[1])
