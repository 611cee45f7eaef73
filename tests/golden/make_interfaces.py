"""Records the reference's Fortran interfaces that the drop-in modules keep (tests/golden/reference_interfaces.json).

Usage: python tests/golden/make_interfaces.py [path to the reference's src directory]
Reads the reference's sources as text (nothing is compiled or run): for every public procedure of module_bse and
module_slepc_solver and the scalar routines whose GPU versions keep their argument lists (eigsys, hlm, optsp,
optdiel and the module_coulomb potentials), the procedure kind, the dummy-argument names in order and each dummy's
type, kind and rank; and the module_bse procedures main.F90 calls.
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

from fortran_decls import logical_lines, procedures  # noqa: E402

SRC = sys.argv[1] if len(sys.argv) > 1 else "/root/reference/src"
MODULES = {"module_bse.F90": None, "module_slepc_solver.F90": ["slepc_solver", "slepc_check_results"],
           "module_hamiltonian.F90": ["eigsys"], "module_optics.F90": ["hlm", "optsp", "optdiel"],
           "module_coulomb.F90": ["v2dk", "vcoul", "v3diel", "v2dt", "v0dt", "v2dt2", "v2drk", "v2dohono", "v1dt"]}
# module_bse's public procedures (its whole contains section; excwf*/exclft/the unused dielbse variants are
# internal helpers of the workflows and are left out)
BSE_PUBLIC = ["matrizelbse", "dielbsev", "dielbsep", "bsedielraw", "bsedielrawpol", "bsebnds", "bsebndstemp",
              "bsesolver", "bsesolvertemp", "lifetime", "lifetimepol", "spoptprop", "spoptproppol", "bseoptprop",
              "bseoptproppol", "spdielraw", "spdielrawpol", "spoptpolbz", "spoptics"]


def main():
    out = {"procedures": {}, "main_calls": []}
    for f, names in MODULES.items():
        procs = procedures(open(os.path.join(SRC, f), errors="replace").read())
        for n in names or BSE_PUBLIC:
            pr = procs[n]
            out["procedures"][n] = {"module": f[:-4], "kind": pr["kind"], "result": pr["result"], "args": pr["args"],
                                    "types": pr["types"]}
    calls = set()
    for ln in logical_lines(open(os.path.join(SRC, "main.F90"), errors="replace").read()):
        m = re.match(r"^\s*(?:if\s*\(.*\)\s*)?call\s+(\w+)", ln, re.I)
        if m and m.group(1).lower() in BSE_PUBLIC:
            calls.add(m.group(1).lower())
    out["main_calls"] = sorted(calls)
    with open(os.path.join(HERE, "reference_interfaces.json"), "w") as fh:
        json.dump(out, fh, indent=1, sort_keys=True)
        fh.write("\n")
    print(len(out["procedures"]), "procedures,", len(out["main_calls"]), "module_bse calls in main.F90")


if __name__ == "__main__":
    main()
