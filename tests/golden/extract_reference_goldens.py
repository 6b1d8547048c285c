"""Extract the reference's golden values for the two-site path into a fixture.

Reads the reference test sources as text (nothing is compiled or run) and
writes ``reference_goldens.json`` next to this script:

* golden ground-state energies and tolerances of the two-site VMPS tests
  (``tests/test_algorithm/test_two_site_update_finite_vmps.cc``) and the
  FiniteDMRG tests (``tests/test_algorithm/test_finite_dmrg.cc``) for the models
  the oracle builds (Ising, Heisenberg 1D/2D, Hubbard 2x2);
* the MATLAB known answers of ``TridiagExpme1Solver``
  (``tests/test_algorithm/test_lanczos_expmv_solver.cc:70-109``);
* the TDVP free-fermion ground-state energy
  (``tests/test_algorithm/test_two_site_finite_tdvp.cc``);
* the entanglement entropies of the N = 6 Heisenberg ground state, bond by
  bond (``tests/test_one_dim_tn/test_finite_mps/test_finite_mps.cc:304-333``);
* the fermionic two-site VMPS energies (free fermions N = 8, t-J 1D and 2D,
  ``tests/test_algorithm/test_fermion_two_site_update_finite_vmps.cc:80-270``)
  with their sweep parameters and initial product states;
* the two-site VMPS energy of the t-J model with a Rashba term
  (``tests/test_algorithm/test_two_site_update_finite_vmps.cc:627-751``);
* the two-site VMPS energy of the Kondo insulator double chain
  (``tests/test_algorithm/test_two_site_update_finite_vmps.cc:976-1084``;
  initial state i % 2);
* the FiniteDMRG energies of the t-J model (1D, 2D) and the 2 x 2 Hubbard
  model (``tests/test_algorithm/test_finite_dmrg.cc:484-835``);
* the FiniteDMRG energy of the J-K-Gamma model without symmetry
  (``tests/test_algorithm/test_finite_dmrg.cc:346-444``; its initial state
  alternates up and down from site 0).

Usage: python tests/golden/extract_reference_goldens.py <reference_root>
"""
import json
import os
import re
import sys

REF = None  # the reference checkout, from the command line
HERE = os.path.dirname(os.path.abspath(__file__))


def read(rel):
    with open(os.path.join(REF, rel)) as f:
        return f.read()


def case_energies(src, case):
    """Energies passed to RunTest*Case inside TEST_F(..., case)."""
    m = re.search(r"TEST_F\(\s*\w+\s*,\s*%s\s*\)(.*?)(?=\nTEST_F|\Z)" % case, src, re.S)
    body = m.group(1)
    out = []
    for mm in re.finditer(r"RunTest\w*Case\((.*?)\);", body, re.S):
        args = [a.strip() for a in mm.group(1).split(",")]
        out.append((args[-2], args[-1]))
    return out


def fixture_case(src, fixture, case):
    """Body of TEST_F(fixture, case)."""
    m = re.search(r"TEST_F\(\s*%s\s*,\s*%s\s*\)(.*?)(?=\nTEST_F|\nTEST\(|\Z)" % (fixture, case),
                  src, re.S)
    return m.group(1)


def sweep_case(body):
    """(energy, tol, sweep-parameter text, initial labels) of the first
    RunTest*Case in a test body."""
    e = re.search(r"RunTest\w*Case\((.*?)\);", body, re.S).group(1)
    args = [a.strip() for a in e.split(",")]
    p = re.search(r"FiniteVMPSSweepParams\((.*?)\);", body, re.S).group(1)
    labs = re.search(r"DirectStateInit\w*\(\s*\w+\s*,\s*\{([^}]*)\}", body)
    return {"energy": float(args[-2]), "tol": float(args[-1]),
            "sweep_params": " ".join(p.split()),
            "labels": [int(x) for x in labs.group(1).split(",")] if labs else None}


def num(s):
    s = s.replace(" ", "")
    if s == "-0.25*(N-1)":
        return -0.25 * 5
    return float(s)


def main():
    global REF
    if len(sys.argv) != 2:
        sys.exit("usage: extract_reference_goldens.py <reference_root>")
    REF = sys.argv[1]
    vmps = read("tests/test_algorithm/test_two_site_update_finite_vmps.cc")
    dmrg = read("tests/test_algorithm/test_finite_dmrg.cc")
    expmv = read("tests/test_algorithm/test_lanczos_expmv_solver.cc")
    tdvp = read("tests/test_algorithm/test_two_site_finite_tdvp.cc")
    goldens = {"source": "text of the reference test files (see script)", "vmps": {}, "dmrg": {}}
    for case in ("1DIsing", "1DHeisenberg", "2DHeisenberg"):
        e = case_energies(vmps, case)
        goldens["vmps"][case] = {"energy": num(e[0][0]), "tol": float(e[0][1])}
    e = case_energies(vmps, "2Dcase")
    goldens["vmps"]["Hubbard2x2"] = {"energy": num(e[0][0]), "tol": float(e[0][1])}
    for case in ("1DIsing", "1DHeisenberg", "2DHeisenberg"):
        try:
            e = case_energies(dmrg, case)
            goldens["dmrg"][case] = {"energy": num(e[0][0]), "tol": float(e[0][1])}
        except Exception:  # noqa: BLE001 - case absent in this file
            pass
    # TridiagExpme1Solver known answers
    cplx = re.compile(r"QLTEN_Complex\(\s*([-0-9.eE]+)\s*,\s*([-0-9.eE]+)\s*\)")
    m1 = re.search(r"matrix2x2_example1\s*=\s*SymmetricTriDiagonalMatrix\(2,\s*\{([^}]*)\},\s*\{([^}]*)\}\)", expmv)
    d1 = re.search(r"delta1\s*=\s*([-0-9.]+)", expmv)
    r1 = re.search(r"res_example1\[2\]\s*=\s*\{(.*?)\};", expmv, re.S)
    m2 = re.search(r"matrix5x5_example2\s*=\s*SymmetricTriDiagonalMatrix\(\s*5,\s*\{([^}]*)\},\s*\{([^}]*)\}\)", expmv, re.S)
    d2 = re.search(r"delta2\s*=\s*([-0-9.]+)", expmv)
    r2 = re.search(r"res_example2\[5\]\s*\{(.*?)\};", expmv, re.S)
    fl = lambda s: [float(x) for x in s.split(",")]
    goldens["expme1"] = [
        {"a": fl(m1.group(1)), "b": fl(m1.group(2)), "delta": float(d1.group(1)),
         "res": [[float(x), float(y)] for x, y in cplx.findall(r1.group(1))]},
        {"a": fl(m2.group(1)), "b": fl(m2.group(2)), "delta": float(d2.group(1)),
         "res": [[float(x), float(y)] for x, y in cplx.findall(r2.group(1))]},
    ]
    gs = re.search(r"(-3\.49395920743493\d*)", tdvp)
    if gs:
        goldens["tdvp_free_fermion_gs"] = float(gs.group(1))
    fmps = read("tests/test_one_dim_tn/test_finite_mps/test_finite_mps.cc")
    ee = re.search(r"ee_list_std\s*=\s*\{([^}]*)\}", fmps)
    ee_tol = re.search(r"EXPECT_NEAR\(ee_list\[i\],\s*ee_list_std\[i\],\s*([0-9.eE-]+)\)", fmps)
    ee_sweep = re.search(r"Test1DHeisenbergEntanglementEntropy.*?FiniteVMPSSweepParams\((.*?)\);",
                         fmps, re.S)
    goldens["ee_heisenberg6"] = {
        "ee": fl(ee.group(1)), "tol": float(ee_tol.group(1)),
        "sweep_params": " ".join(ee_sweep.group(1).split())}
    ferm = read("tests/test_algorithm/test_fermion_two_site_update_finite_vmps.cc")
    goldens["vmps"]["RashbaTJ"] = sweep_case(
        fixture_case(vmps, "TestTwoSiteAlgorithmTjSystem1U1Symm", "RashbaTermCase"))
    goldens["vmps"]["KondoDoubleChain"] = sweep_case(
        fixture_case(vmps, "TestKondoInsulatorSystem", "doublechain"))
    goldens["fermion_vmps"] = {
        "free_fermion8": sweep_case(fixture_case(ferm, "TestTwoSiteAlgorithmSpinlessFermion",
                                                 "1DFreeFermion")),
        "tj1d": sweep_case(fixture_case(ferm, "TestTwoSiteAlgorithmTjSystem2U1Symm", "1DCase")),
        "tj2d": sweep_case(fixture_case(ferm, "TestTwoSiteAlgorithmTjSystem2U1Symm", "2DCase")),
    }
    goldens["dmrg"]["tj1d"] = sweep_case(fixture_case(dmrg, "TestTwoSiteAlgorithmTjSystem2U1Symm",
                                                      "1DCase"))
    goldens["dmrg"]["tj2d"] = sweep_case(fixture_case(dmrg, "TestTwoSiteAlgorithmTjSystem2U1Symm",
                                                      "2DCase"))
    goldens["dmrg"]["Hubbard2x2"] = sweep_case(fixture_case(dmrg, "TestTwoSiteAlgorithmHubbardSystem",
                                                            "2Dcase"))
    kit = re.search(r"TEST\(\s*TestTwoSiteAlgorithmNoSymmetrySpinSystem\s*,\s*"
                    r"2DKitaevComplexCase\s*\)(.*?)(?=\nTEST_F|\nTEST\(|\nstruct|\Z)", dmrg,
                    re.S).group(1)
    e = [a.strip() for a in re.search(r"RunTestDMRGCase\((.*?)\);", kit, re.S).group(1).split(",")]
    par = lambda name: float(re.search(r"double\s+%s\s*=\s*([-0-9.eE]+);" % name, kit).group(1))
    size = re.search(r"size_t\s+Nx\s*=\s*(\d+)\s*,\s*Ny\s*=\s*(\d+);", kit)
    goldens["dmrg_kitaev_gamma"] = {
        "energy": float(e[-2]), "tol": float(e[-1]),
        "sweep_params": " ".join(re.search(r"FiniteVMPSSweepParams\((.*?)\);", kit,
                                           re.S).group(1).split()),
        "J": par("J"), "K": par("K"), "Gm": par("Gm"), "h": par("h"),
        "Nx": int(size.group(1)), "Ny": int(size.group(2))}
    # the noised two-site VMPS (sweep parameters with their noise fields:
    # FiniteVMPSSweepParams(sweeps, Dmin, Dmax, trunc, LanczosParams(err),
    # noises, max_noise, noise_increase, noise_decrease, alpha))
    noise = read("tests/test_algorithm/test_two_site_noise_update_finite_vmps.cc")
    goldens["noise_vmps"] = {}
    for case in ("1DHeisenberg", "2DHeisenberg"):
        body = fixture_case(noise, "TestNoisedTwoSiteAlgorithmSpinSystem", case)
        e = [a.strip() for a in re.search(r"RunTest\w*Case\((.*?)\);", body, re.S)
             .group(1).split(",")]
        p = re.search(r"FiniteVMPSSweepParams\(\s*(\d+)\s*,\s*(\d+)\s*,\s*(\d+)\s*,\s*"
                      r"([-0-9.eE]+)\s*,\s*LanczosParams\(\s*([-0-9.eE]+)\s*\)\s*,\s*"
                      r"std::vector<double>\s*\{([^}]*)\}([^;]*)\);", body, re.S)
        extra = [float(x) for x in re.findall(r"[-0-9.]+(?:[eE][-+]?[0-9]+)?", p.group(7))]
        names = ["max_noise", "noise_increase", "noise_decrease", "alpha"]
        goldens["noise_vmps"][case] = {
            "energy": float(e[-2]), "tol": float(e[-1]), "sweeps": int(p.group(1)),
            "Dmin": int(p.group(2)), "Dmax": int(p.group(3)), "trunc_err": float(p.group(4)),
            "lanczos_error": float(p.group(5)),
            "noises": [float(x) for x in p.group(6).split(",")],
            **dict(zip(names, extra))}
    with open(os.path.join(HERE, "reference_goldens.json"), "w") as f:
        json.dump(goldens, f, indent=1)
    print(json.dumps(goldens, indent=1))


if __name__ == "__main__":
    main()
