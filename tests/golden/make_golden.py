"""Extracts the reference's own known-answer values for the hot path from its
Julia test files (read as text) into reference_kats.json.

Run from the repository root, giving the path of a QuSpin.jl checkout:
    python tests/golden/make_golden.py <path-to-QuSpin.jl>
The JSON it writes is committed; tests never read the reference at run time.
"""
import json
import os
import re
import sys


def read(root, rel):
    with open(os.path.join(root, rel)) as f:
        return f.read()


def floats(text):
    return [float(x) for x in re.findall(r"-?\d+\.\d+(?:e-?\d+)?", text)]


def main(root):
    kats = {}
    src = read(root, "test/unit/basis_spin_basis_1d.jl")
    m = re.search(r"Set\(states\(basis\)\) == Set\(UInt64\[([0-9, ]+)\]\)", src)
    kats["spin_basis_1d_L4_nup2_states"] = {
        "source": "test/unit/basis_spin_basis_1d.jl:14",
        "L": 4, "nup": 2, "pauli": False,
        "states": sorted(int(x) for x in m.group(1).split(",")),
    }
    rt = read(root, "test/runtests.jl")
    m = re.search(r'@testset "XXZ spectrum" begin(.*?)\nend', rt, re.S)
    block = m.group(1)
    ev = re.search(r"@test eigvals\(H\) ≈ \[(.*?)\]", block, re.S).group(1)
    tr = re.search(r"@test tr\(Matrix\(H\)\) ≈ (-?[0-9.]+)", block).group(1)
    fro = re.search(r"@test norm\(Matrix\(H\)\) ≈ ([0-9.]+)", block).group(1)
    kats["xxz_L4_spectrum"] = {
        "source": "test/runtests.jl:599-620",
        "L": 4, "nup": 2, "pauli": False,
        "terms": [["+-", "jxy/2", [[i, i + 1] for i in range(1, 4)]],
                  ["-+", "jxy/2", [[i, i + 1] for i in range(1, 4)]],
                  ["zz", "1.0", [[i, i + 1] for i in range(1, 4)]],
                  ["z", "inv(sqrt(3.0))", [[i] for i in range(1, 5)]]],
        "jxy": "sqrt(2.0)",
        "eigenvalues": floats(ev),
        "trace": float(tr),
        "frobenius": float(fro),
        "atol": 1e-12,
    }
    m = re.search(r'@testset "QuantumLinearOperator protocol" begin(.*?)\nend', rt, re.S)
    block = m.group(1)
    assert "SpinBasis1D(3; nup=1, pauli=false)" in block
    assert 'OperatorTerm("+-", [(0.7, 1, 2), (0.4, 2, 3)])' in block
    assert 'OperatorTerm("z", [(0.2, 1), (-0.3, 3)])' in block
    assert "diagonal=[0.1, -0.2, 0.3]" in block
    assert "mul!(destination, operator, vector, 1.25, -0.5)" in block
    kats["qlo_protocol_L3"] = {
        "source": "test/runtests.jl:842-894",
        "L": 3, "nup": 1, "pauli": False,
        "terms": [["+-", [[0.7, 1, 2], [0.4, 2, 3]]], ["-+", [[0.7, 1, 2], [0.4, 2, 3]]],
                  ["z", [[0.2, 1], [-0.3, 3]]]],
        "diagonal": [0.1, -0.2, 0.3],
        "vector_unnormalized": [[1, 0], [0, 2], [-0.5, 0]],
        "destination": [[0.25, 0], [0, -0.5], [0.75, 0]],
        "alpha": 1.25, "beta": -0.5,
        "atol": 3e-16, "eigsh_k": 2, "eigsh_atol": 2e-14,
    }
    m = re.search(r'@testset "Parallel exponential action protocol" begin(.*?)\nend', rt, re.S)
    block = m.group(1)
    assert "generator = [0.0 -1.0; 1.0 0.0]" in block
    assert "ExpmMultiplyParallel(generator, 0.25)" in block
    kats["expm_rotation_2x2"] = {
        "source": "test/runtests.jl:198-213",
        "generator": [[0.0, -1.0], [1.0, 0.0]], "a": 0.25,
        "expected": "[cos(0.25), sin(0.25)]", "atol": 3e-16,
    }
    cg = read(root, "test/completeness_gaps.jl")
    m = re.search(r'@testset "matrix-free Krylov paths" begin(.*?)\nend', cg, re.S)
    block = m.group(1)
    assert "OperatorTerm(\"zz\", [(0.9, sites...) for sites in bonds])" in block
    kats["matrix_free_krylov_L8"] = {
        "source": "test/completeness_gaps.jl:208-262",
        "L": 8, "nup": 4, "pauli": False,
        "terms": [["zz", 0.9], ["+-", 0.45], ["-+", 0.45]],
        "times": [0.0, 0.17, 0.83], "expm_a": [0.0, -0.37],
        "matvec_atol": 3e-14, "eigsh_atol": 3e-11, "evolve_atol": 3e-11, "norm_atol": 3e-12,
    }
    oa = read(root, "test/operators_algorithm_regressions.jl")
    assert "translation_basis = SpinBasis1D(\n            8;" in oa
    kats["translation_sector_L8"] = {
        "source": "test/operators_algorithm_regressions.jl:128-167",
        "L": 8, "nup": 4, "pauli": False, "kblock": 0,
        "terms": [["+-", 0.5], ["-+", 0.5], ["zz", 0.9]],
        "atol": 4e-14,
    }
    kats["unchecked_symmetric_qlo"] = {
        "source": "test/operators_algorithm_regressions.jl:106-126",
        "L": 4, "nup": 2, "pauli": False, "kblock": 0,
        "terms": [["z", [[0.7, 1]]]], "atol": 2e-14,
    }
    kats["physical_sectors_L4"] = {
        "source": "test/completeness_gaps.jl:77-124",
        "L": 4, "nup": 2, "pauli": False,
        "terms": [["zz", 1.0], ["+-", 0.5], ["-+", 0.5]], "atol": 2e-12,
    }
    m = re.search(r'@testset "Operator algebra and Krylov tools" begin(.*?)\nend', rt, re.S)
    block = m.group(1)
    rows = re.search(r"A = \[\n(.*?)\n    \]", block, re.S).group(1)
    A = [[float(x) for x in row.split()] for row in rows.strip().split("\n")]
    B = floats(re.search(r"B = Diagonal\(\[(.*?)\]\)", block).group(1))
    v0 = [float(x) for x in re.search(r"v0 = \[(.*?)\]", block).group(1).split(",")]
    assert "lanczos_full(A, v0, 3)" in block and "lanczos_iter(A, v0, 3)" in block

    def after(pattern):
        t = re.search(pattern, block, re.S)
        return floats(t.group(1)), float(t.group(2))
    E, E_atol = after(r"@test E ≈ \[(.*?)\] atol=([0-9.e-]+)")
    coeff = [float(x) for x in re.search(r"lin_comb_Q_T\(\[(.*?)\], Q_T\)", block).group(1).split(",")]
    lc, lc_atol = after(r"lin_comb_Q_T\(\[.*?\], Q_T\) ≈\s*\[(.*?)\] atol=([0-9.e-]+)")
    ea = float(re.search(r"expm_lanczos\(E, V, Q_T; a=(-?[0-9.]+)\)", block).group(1))
    ex, ex_atol = after(r"expm_lanczos\(E, V, Q_T; a=-?[0-9.]+\) ≈\s*\[(.*?)\] atol=([0-9.e-]+)")
    betas = floats(re.search(r"beta = \[(.*?)\]", block).group(1))
    fi, fi_atol = after(r"@test ftlm_identity ≈ \[(.*?)\] atol=([0-9.e-]+)")
    fb, fb_atol = after(r'@test ftlm\["B"\] ≈ \[(.*?)\] atol=([0-9.e-]+)')
    lb, lb_atol = after(r'@test ltlm\["B"\] ≈ \[(.*?)\] atol=([0-9.e-]+)')
    kats["krylov_tools_4x4"] = {
        "source": "test/runtests.jl:130-172",
        "A": A, "B_diagonal": B, "v0": v0, "m": 3,
        "E": E, "E_atol": E_atol, "orthonormal_atol": 2e-15,
        "lin_comb_coeff": coeff, "lin_comb": lc, "lin_comb_atol": lc_atol,
        "expm_a": ea, "expm_lanczos": ex, "expm_atol": ex_atol,
        "iter_atol": 1e-14,
        "beta": betas, "ftlm_identity": fi, "ftlm_identity_atol": fi_atol,
        "ftlm_B": fb, "ftlm_B_atol": fb_atol, "ltlm_B": lb, "ltlm_B_atol": lb_atol,
    }
    m = re.search(r'@testset "Symmetry block tools" begin(.*?)\nend', rt, re.S)
    block = m.group(1)
    assert 'terms = [OperatorTerm("z", [(1.0, 1), (0.5, 2)])]' in block
    assert "blocks = [Dict(:nup => sector) for sector in 0:2]" in block
    assert "psi = normalize(ComplexF64[1, 2, 3, 4])" in block
    assert "times = [0.0, 0.2, 1.0]" in block

    def atol_after(pattern):
        return float(re.search(pattern + r".*?atol=([0-9.e-]+)", block, re.S).group(1))
    kats["block_tools_L2"] = {
        "source": "test/runtests.jl:277-325",
        "L": 2, "pauli": False, "terms": [["z", [[1.0, 1], [0.5, 2]]]],
        "blocks_nup": [0, 1, 2], "psi_unnormalized": [1, 2, 3, 4], "times": [0.0, 0.2, 1.0],
        "evolve_atol": atol_after(r"@test evolve\(blocks_operator, psi, 0.0, times\) ≈"),
        "expm_atol": atol_after(r"@test block_expm\(blocks_operator, psi\) ≈"),
        "grid_first_atol": atol_after(r"@test grid\[:, 1\] ≈ psi"),
        "grid_last_atol": atol_after(r"@test grid\[:, end\] ≈"),
        "grid": {"start": 0.0, "stop": 1.0, "num": 3},
    }
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_kats.json")
    with open(out, "w") as f:
        json.dump(kats, f, indent=1, sort_keys=True)
    print("wrote", out)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path-to-QuSpin.jl>")
    main(sys.argv[1])
