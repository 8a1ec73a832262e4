"""Record the reference's Fortran-callable GPU ABI as a test fixture.

Reads src/gpu/specfem3D_gpu_cuda_method_stubs.c of the SPECFEM3D reference
tree (path = first argument, or the environment variable SPECFEM3D_REFERENCE) — the file that lists
every FC_FUNC_ entry point of the GPU layer with its exact argument list — and
writes tests/golden/reference_gpu_abi.json: {name: {"args": [...], "types": [...]}}.
The ABI contract test compares include/specfem3d_gb300.h against it.
"""
import json
import os
import re
import sys


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SPECFEM3D_REFERENCE", "")
    if not root or not os.path.isdir(root):
        sys.exit("usage: %s <SPECFEM3D source tree> (or set SPECFEM3D_REFERENCE)" % sys.argv[0])
    src = open(os.path.join(root, "src/gpu/specfem3D_gpu_cuda_method_stubs.c")).read()
    out = {}
    for m in re.finditer(r"void\s+FC_FUNC_\(\s*(\w+)\s*,\s*\w+\s*\)\s*\(([^)]*)\)", src):
        args = [a.strip() for a in m.group(2).split(",") if a.strip()]
        names = [re.sub(r"^.*?(\w+)\s*$", r"\1", a.replace("*", " ")) for a in args]
        types = [a[: a.rfind(n)].replace(" ", "") for a, n in zip(args, names)]
        out[m.group(1)] = {"args": names, "types": types}
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_gpu_abi.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=0, sort_keys=True)


if __name__ == "__main__":
    main()
