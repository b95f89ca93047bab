"""Extract the known-answer arrays of GooseFEM's own test-suite (C++ and Python) into a JSON
fixture.

Run in a checkout that has the GooseFEM sources (the fixture is committed, so the
tests never need the sources at run time):

    python tests/golden/make_golden.py /path/to/GooseFEM > tests/golden/reference_kat.json

The script reads the test files as text and copies the brace-initialised literal
arrays named below; it does not compile or execute anything from the reference.
"""

import ast
import json
import os
import re
import sys

# (file, variable, name in the fixture, section marker the variable must follow)
WANTED = [
    ("tests/basic/MeshQuad4.cpp", "coor_", "quad4_5x3_coor", 'SECTION("Regular")'),
    ("tests/basic/MeshQuad4.cpp", "conn_", "quad4_5x3_conn", 'SECTION("Regular")'),
    ("tests/basic/MeshQuad4.cpp", "dofs_", "quad4_5x3_dofs", 'SECTION("Regular")'),
    ("tests/basic/MeshQuad4.cpp", "nodesPeriodic_", "quad4_5x3_nodesPeriodic", 'SECTION("Regular")'),
    ("tests/basic/MeshQuad4.cpp", "dofsPeriodic_", "quad4_5x3_dofsPeriodic", 'SECTION("Regular")'),
    ("tests/basic/MeshQuad4.cpp", "nodesBottomEdge_", "quad4_5x3_nodesBottomEdge", 'SECTION("Regular")'),
    ("tests/basic/MeshQuad4.cpp", "nodesTopEdge_", "quad4_5x3_nodesTopEdge", 'SECTION("Regular")'),
    ("tests/basic/MeshQuad4.cpp", "nodesLeftEdge_", "quad4_5x3_nodesLeftEdge", 'SECTION("Regular")'),
    ("tests/basic/MeshQuad4.cpp", "nodesRightEdge_", "quad4_5x3_nodesRightEdge", 'SECTION("Regular")'),
    ("tests/basic/MeshHex8.cpp", "coor_", "hex8_3x3x3_coor", 'SECTION("Regular")'),
    ("tests/basic/MeshHex8.cpp", "conn_", "hex8_3x3x3_conn", 'SECTION("Regular")'),
    ("tests/basic/MeshHex8.cpp", "dofs_", "hex8_3x3x3_dofs", 'SECTION("Regular")'),
    ("tests/basic/MeshHex8.cpp", "nodesFront_", "hex8_3x3x3_nodesFront", 'SECTION("Regular")'),
    ("tests/basic/MeshHex8.cpp", "nodesBack_", "hex8_3x3x3_nodesBack", 'SECTION("Regular")'),
    ("tests/basic/MeshHex8.cpp", "nodesPeriodic_", "hex8_3x3x3_nodesPeriodic", 'SECTION("Regular")'),
    ("tests/basic/MeshHex8.cpp", "dofsPeriodic_", "hex8_3x3x3_dofsPeriodic", 'SECTION("Regular")'),
    ("tests/basic/MatrixDiagonal.cpp", "a", "quad4_2x2_lumped_mass", 'SECTION("assemble")'),
    ("tests/basic/MatrixDiagonalPartitioned.cpp", "a", "quad4_2x2_lumped_mass_partitioned",
     'SECTION("assemble")'),
    ("tests/basic/Mesh.cpp", "ret", "quad4_3x3_coordination", 'SECTION("coordination")'),
]


def _literal(text, start):
    """Return the balanced {...} literal that begins at or after ``start``."""
    i = text.index("{", start)
    depth = 0
    for j in range(i, len(text)):
        if text[j] == "{":
            depth += 1
        elif text[j] == "}":
            depth -= 1
            if depth == 0:
                return text[i:j + 1]
    raise ValueError("unbalanced literal")


def _to_json(lit):
    s = lit.replace("{", "[").replace("}", "]")
    s = re.sub(r"(\d)\.(?!\d)", r"\1.0", s)  # "0." -> "0.0"
    s = re.sub(r",\s*\]", "]", s)
    return json.loads(s)


def extract(root):
    out = {}
    for rel, var, key, section in WANTED:
        with open(os.path.join(root, rel)) as f:
            text = f.read()
        s0 = text.index(section)
        m = re.compile(r"\b" + re.escape(var) + r"\s*=\s*\{").search(text, s0)
        if m is None:
            raise KeyError(f"{var} not found in {rel}")
        out[key] = {"source": f"{rel}:{text.count(chr(10), 0, m.start()) + 1}",
                    "value": _to_json(_literal(text, m.start()))}

    # elem2node expectations (tests/basic/Mesh.cpp, SECTION "elem2node"): one vector per node.
    rel = "tests/basic/Mesh.cpp"
    with open(os.path.join(root, rel)) as f:
        text = f.read()
    s0 = text.index('SECTION("elem2node")')
    s1 = text.index("SECTION(", s0 + 10)
    rows = re.findall(r"tonode\[(\d+)\] == std::vector<size_t>\{([^}]*)\}", text[s0:s1])
    e2n = [None] * len(rows)
    for k, vals in rows:
        e2n[int(k)] = [int(v) for v in vals.split(",")]
    out["quad4_3x3_elem2node"] = {"source": f"{rel}:{text.count(chr(10), 0, s0) + 1}",
                                  "value": e2n}

    # the Python test-suite (tests/test_Mesh.py): the literal expected values of four tests on
    # Quad4 Regular(4, 4) with periodic dofs and one on Regular(3, 3), read with ast (parsed,
    # never executed)
    rel = "tests/test_Mesh.py"
    with open(os.path.join(root, rel)) as f:
        tree = ast.parse(f.read())
    wanted_py = {"test_center_of_gravity": "quad4_3x3_center_of_gravity",
                 "test_coordination_dofs": "quad4_4x4_coordination_dofsPeriodic",
                 "test_coordination_node2dof": "quad4_4x4_node2dof",
                 "test_coordination_nodaltyings": "quad4_4x4_nodaltyings",
                 "test_elem2node_periodic": "quad4_4x4_elem2node_periodic"}
    for fn in ast.walk(tree):
        if isinstance(fn, ast.FunctionDef) and fn.name in wanted_py:
            lists = [n for n in ast.walk(fn) if isinstance(n, ast.List)]
            outer = max(lists, key=lambda n: len(ast.dump(n)))  # the largest literal
            out[wanted_py[fn.name]] = {"source": f"{rel}:{outer.lineno}",
                                       "value": ast.literal_eval(outer)}
    return out


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    json.dump(extract(root), sys.stdout, indent=0)
    sys.stdout.write("\n")
