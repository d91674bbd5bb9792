"""Regenerates the golden fixtures of this directory from the reference's own tests.

Run as `python make_golden.py <path of the CheMPS2 checkout>` (or with REFERENCE set to
that path); the outputs are committed so that the tests never read the reference at run
time.

  * N2.STO3G.FCIDUMP    copied from tests/matrixelements/N2.STO3G.FCIDUMP (the input of
                        the reference's tests/test1.cpp.in and tests/test5.cpp.in)
  * H2O.631G.FCIDUMP    copied from tests/matrixelements/H2O.631G.FCIDUMP (the input of
                        the reference's tests/test2.cpp.in, DMRG against FCI; the FCI takes
                        about 15 minutes on 8 threads, so its test runs on request only)
  * CH4.STO3G.FCIDUMP   copied from tests/matrixelements/CH4.STO3G.FCIDUMP (the input of
                        the reference's tests/test3.cpp.in, which compares DMRG with FCI;
                        its schedule is recorded in golden.json, the FCI energy is computed
                        by the oracle)
  * golden.json         energies the reference's tests assert, parsed from their sources,
                        and the settings of its DMRG-against-FCI tests (tests/test1.cpp.in:
                        N2 STO-3G in six symmetry sectors; tests/test3.cpp.in: CH4 STO-3G):
                        tests/test5.cpp.in (N2 STO-3G ground and two excited states,
                        D = 1000) and
                        tests/test12.cpp.in (the BCS pairing model, L = 8)
"""
from __future__ import annotations

import json
import os
import re
import shutil
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent


def main(reference: Path) -> None:
    tests = reference / "tests"
    shutil.copyfile(tests / "matrixelements" / "N2.STO3G.FCIDUMP", HERE / "N2.STO3G.FCIDUMP")
    shutil.copyfile(tests / "matrixelements" / "CH4.STO3G.FCIDUMP", HERE / "CH4.STO3G.FCIDUMP")
    shutil.copyfile(tests / "matrixelements" / "H2O.631G.FCIDUMP", HERE / "H2O.631G.FCIDUMP")
    t2 = (tests / "test2.cpp.in").read_text()
    t3 = (tests / "test3.cpp.in").read_text()
    t1 = (tests / "test1.cpp.in").read_text()
    t5 = (tests / "test5.cpp.in").read_text()
    t12 = (tests / "test12.cpp.in").read_text()
    e5 = [float(x) for x in re.findall(r"fabs\(\s*Energy\d\s*\+\s*([0-9.]+)\s*\)", t5)]
    e12 = [float(x) for x in re.findall(r"fabs\(\s*Energy\s*\+\s*([0-9.]+)\s*\)", t12)]
    golden = {
        "n2_sto3g": {
            "source": "tests/test5.cpp.in",
            "fcidump": "N2.STO3G.FCIDUMP",
            "group": 7,
            "two_s": 0,
            "n": 14,
            "irrep": 0,
            "reorder": "d2h",
            "schedule": [[1000, 1e-12, 100, 0.0, 1e-5]],
            "energy": -e5[0],
            # the two excited states of the same test: newExcitation(20.0) twice
            "excited_eshift": 20.0,
            "excited_energies": [-e5[1], -e5[2]],
            "tolerance": 1e-8,
        },
        "bcs_l8": {
            "source": "tests/test12.cpp.in",
            "eps": [-3.5, -2.5, -1.5, -0.5, 0.5, 1.5, 2.5, 3.5],
            "g": -1.0,
            "power": 0.0,
            "two_s": 0,
            "n": 8,
            "irrep": 0,
            "schedule": [[100, 1e-10, 10, 0.5, 1e-5], [1000, 1e-10, 10, 0.0, 1e-5]],
            "energy": -e12[0],
            "tolerance": 1e-8,
        },
    }
    # tests/test3.cpp.in: group, particle numbers and the two instructions (D, Econv,
    # sweeps, noise) of its ConvergenceScheme; the Davidson tolerance is the reference's
    # default for DMRG (CheMPS2/include/chemps2/Options.h: DAVIDSON_DMRG_RTOL = 1e-5)
    grp = int(re.search(r"psi4groupnumber\s*=\s*(\d+)", t3).group(1))
    n3 = int(re.search(r"int\s+N\s*=\s*(\d+)", t3).group(1))
    s3 = int(re.search(r"int\s+TwoS\s*=\s*(\d+)", t3).group(1))
    i3 = int(re.search(r"int\s+Irrep\s*=\s*(\d+)", t3).group(1))
    instr = re.findall(r"OptScheme->setInstruction\(\s*(\d+)\s*,\s*(\d+)\s*,\s*([0-9.e+-]+)\s*,\s*(\d+)\s*,"
                       r"\s*([0-9.e+-]+)\s*\)", t3)
    golden["ch4_sto3g"] = {
        "source": "tests/test3.cpp.in",
        "fcidump": "CH4.STO3G.FCIDUMP",
        "group": grp,
        "two_s": s3,
        "n": n3,
        "irrep": i3,
        "schedule": [[int(d), float(e), int(sw), float(nz), 1e-5] for _, d, e, sw, nz in instr],
        "tolerance": 1e-08,
    }
    # tests/test1.cpp.in: N2 STO-3G in six (2S, irrep) sectors, each with its two
    # set_instruction calls (D, Econv, sweeps, noise, Davidson rtol)
    arr = lambda name: [int(x) for x in re.search(name + r"\[\]\s*=\s*\{([^}]*)\}", t1).group(1).split(",")]
    instr1 = re.findall(r"opt_scheme\.set_instruction\(\s*\d+\s*,\s*(\d+)\s*,\s*([0-9.e+-]+)\s*,\s*(\d+)\s*,"
                        r"\s*([0-9.e+-]+)\s*,\s*([0-9.e+-]+)\s*\)", t1)
    golden["n2_sto3g_sectors"] = {
        "source": "tests/test1.cpp.in",
        "fcidump": "N2.STO3G.FCIDUMP",
        "group": int(re.search(r"psi4groupnumber\s*=\s*(\d+)", t1).group(1)),
        "n": int(re.search(r"Nelec\s*=\s*(\d+)", t1).group(1)),
        "two_s": arr("TwoS"),
        "irreps": arr("Irreps"),
        "schedule": [[int(d), float(e), int(sw), float(nz), float(rt)] for d, e, sw, nz, rt in instr1],
        "tolerance": 1e-08,
    }
    # tests/test2.cpp.in: H2O 6-31G, same layout as test3
    instr2 = re.findall(r"OptScheme->setInstruction\(\s*(\d+)\s*,\s*(\d+)\s*,\s*([0-9.e+-]+)\s*,\s*(\d+)\s*,"
                        r"\s*([0-9.e+-]+)\s*\)", t2)
    golden["h2o_631g"] = {
        "source": "tests/test2.cpp.in",
        "fcidump": "H2O.631G.FCIDUMP",
        "group": int(re.search(r"psi4groupnumber\s*=\s*(\d+)", t2).group(1)),
        "two_s": int(re.search(r"TwoS\s*=\s*(\d+)", t2).group(1)),
        "n": int(re.search(r"\bN\s*=\s*(\d+)", t2).group(1)),
        "irrep": int(re.search(r"Irrep\s*=\s*(\d+)", t2).group(1)),
        "schedule": [[int(d), float(e), int(sw), float(nz), 1e-5] for _, d, e, sw, nz in instr2],
        "tolerance": 1e-08,
    }
    (HERE / "golden.json").write_text(json.dumps(golden, indent=2) + "\n")


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("REFERENCE")
    if not ref:
        sys.exit("usage: make_golden.py <path of the CheMPS2 checkout> (or set REFERENCE)")
    main(Path(ref))
