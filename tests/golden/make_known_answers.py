"""Writes tests/golden/known_answers.json.

The values are the assertions of GalerkinToolkit.jl's own test-suite (each
entry names its file:line in the reference tree); they are copied as data,
not computed, because the Julia reference cannot run here.  Run this script
from the repository root to regenerate the fixture after editing the table.
"""
import json
import os

KNOWN = {
    "_about": ("Known answers held by GalerkinToolkit.jl v0.6.3's own test-suite for the assembly path, "
               "transcribed with their file:line. The Julia reference cannot run in this environment (no Julia "
               "toolchain), so these asserted values are what pins the CPU oracle; see "
               "tests/golden/make_known_answers.py."),
    "q2_unit_square_boundary_dirichlet": {
        "source": "test/assembly_tests.jl:44-73",
        "mesh": "GT.mesh(GT.unit_n_cube(Val(2))) == cartesian_mesh((0,1,0,1),(1,1))",
        "order": 2, "num_free_dofs": 1, "num_dirichlet_dofs": 8},
    "q1_2x2_sum_of_load_vector": {
        "source": "test/problems_tests.jl:12-53", "mesh": "cartesian_mesh((0,1,0,1),(2,2))",
        "order": 1, "degree": 2, "sum_b": 1.0},
    "q1_2x2_sum_of_mass_matrix": {
        "source": "test/problems_tests.jl:54-56, refill via update_matrix! at :70-77",
        "mesh": "cartesian_mesh((0,1,0,1),(2,2))", "order": 1, "degree": 2, "sum_A": 1.0},
    "integral_x_plus_y_on_0_2_square": {
        "source": "test/integration_tests.jl:45-77", "mesh": "cartesian_mesh((0,2,0,2),(8,8))",
        "degree": 2, "int_x_plus_y": 8.0, "int_one": 4.0},
    "quadrature_weight_sums": {
        "source": "test/space_tests.jl:183-189, :272-279", "square_degree_2": 1.0, "cube_degree_4": 1.0},
    "q1_square_reference_faces": {
        "source": "test/space_tests.jl:283-287",
        "face_nodes_1": [[1, 2], [3, 4], [1, 3], [2, 4]], "face_nodes_0": [[1], [2], [3], [4]]},
    "patch_tests_u_equals_x_plus_y": {
        "tol": 1e-10,
        "cases": [
            {"source": "test/assembly_tests.jl:44-118", "box": [0, 1, 0, 1], "cells": [1, 1], "order": 2},
            {"source": "test/problems_tests.jl:85-100", "box": [0, 1, 0, 1], "cells": [2, 2], "order": 1},
            {"source": "test/problems_ext_tests.jl:117-144", "box": [0, 1, 0, 1], "cells": [10, 10], "order": 1},
            {"source": "GalerkinToolkitExamples/test/poisson_tests.jl:7-27", "box": [0, 2, 0, 2], "cells": [2, 2],
             "order": 2},
        ]},
}

if __name__ == "__main__":
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "known_answers.json")
    with open(out, "w") as f:
        json.dump(KNOWN, f, indent=2)
        f.write("\n")
    print(out)
