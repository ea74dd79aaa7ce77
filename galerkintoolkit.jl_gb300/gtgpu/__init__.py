"""gtgpu -- GB300-native finite-element assembly and solve with the
GalerkinToolkit.jl problem-level API (assemble_matrix / assemble_vector /
linear problem + solve) over hand-written sm_103a CUDA kernels."""
from ._lib import GTError, load  # noqa: F401
from .api import (Context, DeviceArray, DiscreteField, Domain, Form, LinearProblem, Matrix, Polynomial, Source,  # noqa: F401
                  Space, lognormal_cells_device,
                  assemble_boundary_vector, assemble_matrix, assemble_matrix_and_vector, assemble_vector, boundary,
                  default_context, device_mesh, elasticity, h1_error, integrate, interior, interpolate_dirichlet,
                  l2_error, lagrange_space, laplacian, linear_problem, mass, num_dirichlet_dofs, num_free_dofs, solve,
                  source, update_matrix, update_matrix_and_vector, dirichlet_field, solution_field, solution_field_inplace,
                  zero_dirichlet_field)
from .mesh import Mesh, cartesian_mesh, jitter_interior_nodes, keyed_uniform, lognormal_cells  # noqa: F401
