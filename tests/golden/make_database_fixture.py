"""Record the order of the records in the reference's solver database as a test
fixture.

Reads generate_databases/save_arrays_solver.F90 of a SPECFEM3D source tree (path =
first argument, or the environment variable SPECFEM3D_REFERENCE), takes the
subroutine save_arrays_solver_mesh and lists, in source order, the variables of
every `write(IOUT) <variables>` statement (including one-line `if (...) write`),
with the guard conditions of the enclosing if blocks; writes
tests/golden/reference_database_records.json.  The database test checks that the
records specfem3d_gb300.databases writes follow this order under the same names.
"""
import json
import os
import re
import sys


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SPECFEM3D_REFERENCE", "")
    if not root or not os.path.isdir(root):
        sys.exit("usage: %s <SPECFEM3D source tree> (or set SPECFEM3D_REFERENCE)" % sys.argv[0])
    src = open(os.path.join(root, "src/generate_databases/save_arrays_solver.F90")).read().splitlines()
    start = next(i for i, l in enumerate(src) if re.match(r"\s*subroutine save_arrays_solver_mesh\b", l))
    end = next(i for i, l in enumerate(src) if re.match(r"\s*end subroutine save_arrays_solver_mesh\b", l))
    stack, records = [], []
    for lineno in range(start, end):
        line = src[lineno].split("!")[0].strip()
        if not line:
            continue
        m = re.match(r"if\s*\((.*)\)\s*then$", line)
        if m:
            stack.append(m.group(1).strip())
            continue
        if re.match(r"else\s*if\s*\(", line) or line == "else":
            stack[-1] = "not(" + stack[-1] + ")" + ("" if line == "else" else " and " + line)
            continue
        if re.match(r"end\s*if$", line):
            stack.pop()
            continue
        m = re.match(r"(?:if\s*\((.*)\)\s*)?write\s*\(\s*IOUT\s*\)\s*([\w\s,]+?)\s*$", line)
        if m:
            guards = list(stack) + ([m.group(1).strip()] if m.group(1) else [])
            name = ",".join(v.strip() for v in m.group(2).split(","))
            records.append({"name": name, "line": lineno + 1, "guards": guards})
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_database_records.json")
    with open(path, "w") as f:
        json.dump({"source": "src/generate_databases/save_arrays_solver.F90", "subroutine": "save_arrays_solver_mesh",
                   "records": records}, f, indent=1)
    print(f"{len(records)} records -> {path}")


if __name__ == "__main__":
    main()
