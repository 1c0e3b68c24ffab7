"""Generate tests/golden/kat.json: known-answer values for the LLG path.

The reference (OCaml + Python 2 + PETSc + SUNDIALS) cannot run here and its
tree ships no golden vectors, so these fixtures are derived independently of
both the oracle and the product:

* mesh counts of the Kuhn-split box from closed-form combinatorics
  (nodes, tets, edges, P1 nonzeros N + 2E, boundary nodes, outer faces);
* simulation-unit material coefficients computed with plain arithmetic from
  the formulas of interface/nmag/main.py:419-465 and the constants of
  interface/nsim/si_units/si.py, with the unit scales of main.py:188-196.

Run:  python tests/golden/make_golden.py
"""
import json
import math
import os


def box_counts(nx, ny, nz):
    N = (nx + 1) * (ny + 1) * (nz + 1)
    T = 6 * nx * ny * nz
    axis = nx * (ny + 1) * (nz + 1) + (nx + 1) * ny * (nz + 1) + (nx + 1) * (ny + 1) * nz
    face_diag = nx * ny * (nz + 1) + nx * (ny + 1) * nz + (nx + 1) * ny * nz
    body = nx * ny * nz
    E = axis + face_diag + body
    interior = max(nx - 1, 0) * max(ny - 1, 0) * max(nz - 1, 0)
    return {"nodes": N, "tets": T, "edges": E, "nnz": N + 2 * E, "boundary_nodes": N - interior,
            "outer_faces": 4 * (nx * ny + ny * nz + nx * nz)}


def su_coefficients(Ms_si, A_si, alpha, gamma_si, norm_si=0.1e12):
    # simulation units: A=1e-3, kg=1e-27, m=1e-9, s=1e-12
    su_Ms = Ms_si / (1e-3 / 1e-9)                 # A/m
    su_A = A_si / (1e-27 * 1e-9 / 1e-24)          # J/m = kg m s^-2
    su_mu0 = 4e-7 * math.pi / (1e-27 * 1e-9 / (1e-24 * 1e-6))  # N/A^2 = kg m s^-2 A^-2
    su_gamma = gamma_si / (1e-9 / (1e-3 * 1e-12))  # m/(A s)
    su_norm = norm_si / (1.0 / 1e-12)
    g2ll = 1.0 / (1.0 + alpha * alpha)
    c1 = -su_gamma * g2ll
    return {"su_Ms": su_Ms, "su_A": su_A, "su_mu0": su_mu0, "su_gamma": su_gamma,
            "exch_prefactor": 2.0 * su_A / (su_mu0 * su_Ms), "C1": c1, "C2": c1 * alpha, "C3": su_norm,
            "one_degree_per_ns": (math.pi / 180.0 / 1e-9) * 1e-12}


def main():
    out = {
        "cube_10": box_counts(10, 10, 10),
        "film_200x50x2": box_counts(200, 50, 2),
        "box_4x3x2": box_counts(4, 3, 2),
        "particles": {str(n): box_counts(n, n, n) for n in (4, 8, 20)},
        "permalloy_alpha05": su_coefficients(8.6e5, 1.3e-11, 0.5, 2.211e5),
        "permalloy_alpha002": su_coefficients(8.6e5, 1.3e-11, 0.02, 2.211e5),
        "nmag_default_material": su_coefficients(0.86e6, 1.3e-11, 0.5, 2.210173e5),
    }
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "kat.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    print(path)


if __name__ == "__main__":
    main()
