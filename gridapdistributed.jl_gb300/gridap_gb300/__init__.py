"""GB300 assembly-and-solve backend for GridapDistributed-style Cartesian problems.

``distributed`` mirrors the reference's Julia API over the C ABI in
``include/gdgpu.h``; ``_lib`` is the ctypes binding of ``libgdgpu.so``.
"""
from . import _lib
from .distributed import (AffineFEOperator, AssembledPVector, Boundary, CartesianDiscreteModel, FEFunction,
                          FESpace, FullyAssembledRows, GB300Backend, Measure, PSparseMatrix, PVector,
                          ReferenceFE, SparseMatrixAssembler, SubAssembledRows, TestFESpace,
                          Triangulation, TrialFESpace, VectorValue, allocate_matrix, allocate_matrix_and_vector,
                          allocate_vector, assemble_matrix, assemble_matrix_, assemble_matrix_and_vector,
                          assemble_matrix_and_vector_, assemble_vector, assemble_vector_, collect_cell_matrix,
                          collect_cell_matrix_and_vector, collect_cell_vector, get_dirichlet_dof_values,
                          integral_boundary_source, integral_elasticity, integral_grad_grad,
                          integral_source, interpolate, interpolate_dirichlet, interpolate_dirichlet_,
                          interpolate_everywhere, interpolate_everywhere_, l2_error, lagrangian,
                          quadrature_points, solve, with_gb300, zero_dirichlet_values, zero_free_values)
from .dg import Skeleton, integral_sipg, integral_sipg_source
from .multifield import (BlockMultiFieldStyle, BlockPMatrix, BlockPVector, ConsecutiveMultiFieldStyle,
                         MultiFieldFESpace, integral_multifield, integral_multifield_source,
                         restrict_to_field)

__all__ = [n for n in dir() if not n.startswith("_")]
