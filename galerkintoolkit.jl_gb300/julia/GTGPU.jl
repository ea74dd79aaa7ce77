"""
    GTGPU

Julia binding of `libgtgpu.so` (C ABI in `include/gtgpu.h`): the GB300
replacement of GalerkinToolkit's problem-level assembly and solve calls.
It keeps GT's calling shape (`assemble_matrix(a, T, U, V)`,
`assemble_vector(l, T, V)`, `update_matrix!`, linear problem + solve) for the
supported forms and returns a `SparseMatrixCSC{T,Int32}` on download.

Not exercised in this repository's test-suite (no Julia toolchain in the
build image); the Python binding in `gtgpu/_lib.py` binds the same symbols.
"""
module GTGPU

using SparseArrays

const LIB = get(ENV, "GTGPU_LIB", joinpath(@__DIR__, "..", "_build", "libgtgpu.so"))

const GT_QUAD4, GT_HEX8, GT_TET4 = Cint(1), Cint(2), Cint(3)
const GT_LAPLACE, GT_MASS, GT_ELASTICITY = Cint(1), Cint(2), Cint(3)
const GT_FP64, GT_FP32, GT_MIXED = Cint(0), Cint(1), Cint(2)
const GT_SOLVE_FP64, GT_SOLVE_IR, GT_SOLVE_FP32 = Cint(0), Cint(1), Cint(2)

struct SolveInfo
    iterations::Int32
    outer_iterations::Int32
    rel_residual::Float64
    fp64_iterations::Int32
    reserved::Int32
end

function check(ctx, st)
    st == 0 && return nothing
    msg = unsafe_string(ccall((:gt_last_error, LIB), Cstring, (Ptr{Cvoid},), ctx))
    error("gtgpu status $st: $msg")
end

mutable struct Context
    h::Ptr{Cvoid}
end
function Context(device::Integer=0)
    r = Ref{Ptr{Cvoid}}(C_NULL)
    st = ccall((:gt_ctx_create, LIB), Cint, (Cint, Ptr{Ptr{Cvoid}}), device, r)
    st == 0 || error("gt_ctx_create failed ($st)")
    c = Context(r[])
    finalizer(c -> ccall((:gt_ctx_destroy, LIB), Cint, (Ptr{Cvoid},), c.h), c)
    c
end

struct Mesh
    ctx::Context
    h::Ptr{Cvoid}
end

"""
    Mesh(ctx, cell_type, coords::Matrix{Float64} (D x nnodes), cell_nodes::Matrix{Int32} (nv x ncells),
         corners, bfaces (nfv x nb), bface_group, bedges (2 x ne))

Uploads a GT mesh (1-based ids, the layout of GT.node_coordinates / GT.face_nodes).
"""
function Mesh(ctx::Context, cell_type, coords, cell_nodes, corners, bfaces, bface_group, bedges)
    r = Ref{Ptr{Cvoid}}(C_NULL)
    st = ccall((:gt_mesh_create, LIB), Cint,
               (Ptr{Cvoid}, Cint, Int64, Ptr{Float64}, Int64, Ptr{Int32}, Int64, Ptr{Int32}, Int64, Ptr{Int32},
                Ptr{Int32}, Int64, Ptr{Int32}, Ptr{Ptr{Cvoid}}),
               ctx.h, cell_type, size(coords, 2), coords, size(cell_nodes, 2), cell_nodes, length(corners), corners,
               size(bfaces, 2), bfaces, bface_group, size(bedges, 2), bedges, r)
    check(ctx.h, st)
    Mesh(ctx, r[])
end

struct Space
    ctx::Context
    h::Ptr{Cvoid}
    num_free_dofs::Int
    num_dirichlet_dofs::Int
end

"""
    lagrange_space(mesh, order; tensor_size=nothing, dirichlet_groups=:boundary)

`dirichlet_groups`: `:boundary`, `nothing`, or a vector of k of "(D-1)-face-k".
"""
function lagrange_space(m::Mesh, order; tensor_size=nothing, dirichlet_groups=:boundary)
    ncomp = tensor_size === nothing ? 1 : only(tensor_size)
    ng, groups = dirichlet_groups === :boundary ? (-1, Int32[]) :
                 dirichlet_groups === nothing ? (0, Int32[]) : (length(dirichlet_groups), Int32.(dirichlet_groups))
    r = Ref{Ptr{Cvoid}}(C_NULL)
    check(m.ctx.h, ccall((:gt_space_create, LIB), Cint, (Ptr{Cvoid}, Cint, Cint, Cint, Ptr{Int32}, Ptr{Ptr{Cvoid}}),
                         m.h, order, ncomp, ng, groups, r))
    info = zeros(Int64, 6)
    check(m.ctx.h, ccall((:gt_space_info, LIB), Cint, (Ptr{Cvoid}, Ptr{Int64}), r[], info))
    Space(m.ctx, r[], info[1], info[2])
end

struct Form
    kind::Cint
    coef::Union{Nothing,Vector{Float64}}
    nu::Float64
end
laplacian(coef=nothing) = Form(GT_LAPLACE, coef, 0.3)
mass(coef=nothing) = Form(GT_MASS, coef, 0.3)
elasticity(E=nothing, nu=0.3) = Form(GT_ELASTICITY, E, nu)
_coef(f::Form) = f.coef === nothing ? C_NULL : f.coef
_prec(::Type{Float64}) = GT_FP64
_prec(::Type{Float32}) = GT_FP32

mutable struct DeviceMatrix
    space::Space
    h::Ptr{Cvoid}
end

"""
    assemble_matrix(a::Form, T, U::Space, V::Space=U) -> SparseMatrixCSC{T,Int32}, cache

Mirrors GT.assemble_matrix(a, T, U, V; reuse=Val(true)).
"""
function assemble_matrix(a::Form, ::Type{T}, U::Space, V::Space=U) where {T}
    U === V || error("trial and test spaces must be the same")
    r = Ref{Ptr{Cvoid}}(C_NULL)
    check(U.ctx.h, ccall((:gt_assemble_matrix, LIB), Cint, (Ptr{Cvoid}, Cint, Ptr{Float64}, Float64, Cint, Ptr{Ptr{Cvoid}}),
                         U.h, a.kind, _coef(a), a.nu, _prec(T), r))
    dm = DeviceMatrix(U, r[])
    finalizer(m -> ccall((:gt_matrix_destroy, LIB), Cint, (Ptr{Cvoid},), m.h), dm)
    download(dm, T), dm
end

function download(dm::DeviceMatrix, ::Type{T}) where {T}
    info = zeros(Int64, 6)
    check(dm.space.ctx.h, ccall((:gt_matrix_info, LIB), Cint, (Ptr{Cvoid}, Ptr{Int64}), dm.h, info))
    n, nnz = info[1], info[2]
    rowptr = zeros(Int64, n + 1)
    colind = zeros(Int32, nnz)
    v64 = T === Float64 ? zeros(Float64, nnz) : C_NULL
    v32 = T === Float32 ? zeros(Float32, nnz) : C_NULL
    check(dm.space.ctx.h, ccall((:gt_matrix_download_csr, LIB), Cint,
                                (Ptr{Cvoid}, Ptr{Int64}, Ptr{Int32}, Ptr{Float64}, Ptr{Float32}), dm.h, rowptr, colind, v64, v32))
    # symmetric pattern and values: CSR rows are CSC columns
    SparseMatrixCSC{T,Int32}(n, n, Int32.(rowptr .+ 1), colind .+ Int32(1), T === Float64 ? v64 : v32)
end

_dmatrix(V::Space, h) = (dm = DeviceMatrix(V, h);
                          finalizer(m -> ccall((:gt_matrix_destroy, LIB), Cint, (Ptr{Cvoid},), m.h), dm); dm)
_ptr_or_null(a) = a === nothing ? C_NULL : a

"""
    assemble_matrix_and_vector(a::Form, f (ncomp), T, V; source_coef=nothing) -> A, b, dm

GT.assemble_matrix_and_vector(a, l, T, U, V) for l(v) = ∫ source_coef f⋅v:
matrix and load vector in one pass (gt_assemble_matrix_and_vector).
"""
function assemble_matrix_and_vector(a::Form, f::AbstractVector, ::Type{T}, V::Space; source_coef=nothing) where {T}
    b = zeros(Float64, V.num_free_dofs)
    r = Ref{Ptr{Cvoid}}(C_NULL)
    check(V.ctx.h, ccall((:gt_assemble_matrix_and_vector, LIB), Cint,
                         (Ptr{Cvoid}, Cint, Ptr{Float64}, Float64, Cint, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
                          Ptr{Ptr{Cvoid}}),
                         V.h, a.kind, _coef(a), a.nu, _prec(T), collect(Float64, f), _ptr_or_null(source_coef), b, r))
    dm = _dmatrix(V, r[])
    download(dm, T), b, dm
end

"""
    linear_problem(dirichlet_values, a::Form, f (ncomp), T, V; source_coef=nothing) -> A, b, dm

GT.PartitionedSolvers_linear_problem(uhd, a, l): A and b with the Dirichlet
lift b -= Ad * dirichlet_values (values in the Dirichlet numbering) in the
same pass (gt_linear_problem).
"""
function linear_problem(dirichlet_values::AbstractVector, a::Form, f::AbstractVector, ::Type{T}, V::Space;
                        source_coef=nothing) where {T}
    b = zeros(Float64, V.num_free_dofs)
    r = Ref{Ptr{Cvoid}}(C_NULL)
    check(V.ctx.h, ccall((:gt_linear_problem, LIB), Cint,
                         (Ptr{Cvoid}, Cint, Ptr{Float64}, Float64, Cint, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
                          Ptr{Float64}, Ptr{Ptr{Cvoid}}),
                         V.h, a.kind, _coef(a), a.nu, _prec(T), collect(Float64, f), _ptr_or_null(source_coef),
                         collect(Float64, dirichlet_values), b, r))
    dm = _dmatrix(V, r[])
    download(dm, T), b, dm
end

"""
    update_matrix_and_vector!(A, b, dm::DeviceMatrix, a::Form, f; source_coef=nothing)

GT.update_matrix_and_vector!: new values and load vector on the assembled
pattern (gt_update_matrix_and_vector).
"""
function update_matrix_and_vector!(A::SparseMatrixCSC{T}, b::Vector{Float64}, dm::DeviceMatrix, a::Form,
                                   f::AbstractVector; source_coef=nothing) where {T}
    check(dm.space.ctx.h, ccall((:gt_update_matrix_and_vector, LIB), Cint,
                                (Ptr{Cvoid}, Cint, Ptr{Float64}, Float64, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
                                dm.h, a.kind, _coef(a), a.nu, collect(Float64, f), _ptr_or_null(source_coef), b))
    copyto!(A.nzval, download(dm, T).nzval)
    A, b
end

"""
    update_matrix!(A, dm::DeviceMatrix, a::Form)   (GT.update_matrix!)
"""
function update_matrix!(A::SparseMatrixCSC{T}, dm::DeviceMatrix, a::Form) where {T}
    check(dm.space.ctx.h, ccall((:gt_update_matrix, LIB), Cint, (Ptr{Cvoid}, Cint, Ptr{Float64}, Float64),
                                dm.h, a.kind, _coef(a), a.nu))
    copyto!(A.nzval, download(dm, T).nzval)
    A
end

"""
    assemble_vector(f::Vector{Float64} (ncomp), T, V; coef=nothing)   (GT.assemble_vector of v -> ∫ coef f⋅v)
"""
function assemble_vector(f::AbstractVector, ::Type{Float64}, V::Space; coef=nothing)
    b = zeros(Float64, V.num_free_dofs)
    check(V.ctx.h, ccall((:gt_assemble_vector, LIB), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
                         V.h, collect(Float64, f), coef === nothing ? C_NULL : coef, b))
    b
end

"""
    assemble_boundary_vector!(b, g::Vector{Float64} (ncomp), V, groups; accumulate=true)

GT.assemble_vector(v -> ∫ g⋅v dΓ) over the boundary faces of the groups k of
"(D-1)-face-k" (`groups === :boundary`: all of them), added to b.
"""
function assemble_boundary_vector!(b::Vector{Float64}, g::AbstractVector, V::Space, groups; accumulate=true)
    ng, gs = groups === :boundary ? (Cint(-1), C_NULL) : (Cint(length(groups)), Int32.(groups))
    check(V.ctx.h, ccall((:gt_assemble_boundary_vector, LIB), Cint,
                         (Ptr{Cvoid}, Cint, Ptr{Int32}, Ptr{Float64}, Ptr{Float64}, Cint),
                         V.h, ng, gs, collect(Float64, g), b, accumulate ? Cint(1) : Cint(0)))
    b
end

const GT_INT_VOLUME, GT_INT_POLY, GT_INT_FIELD, GT_INT_L2_NORM2, GT_INT_L2_ERROR2, GT_INT_H1_ERROR2 = 0, 1, 2, 3, 4, 5

"""
    integrate(V, kind; u_free=nothing, u_dirichlet=nothing, poly=nothing) -> Float64

GT.assemble_scalar for the fixed integrands of `gt_integrate` (e.g. the
squared L2 error `kind = GT_INT_L2_ERROR2` against a quadratic with the 10
coefficients of 1, x, y, z, x², y², z², xy, xz, yz per component).
"""
function integrate(V::Space, kind::Integer; u_free=nothing, u_dirichlet=nothing, poly=nothing)
    r = Ref{Float64}(0.0)
    check(V.ctx.h, ccall((:gt_integrate, LIB), Cint,
                         (Ptr{Cvoid}, Cint, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ref{Float64}),
                         V.h, kind, u_free === nothing ? C_NULL : u_free,
                         u_dirichlet === nothing ? C_NULL : u_dirichlet, poly === nothing ? C_NULL : poly, r))
    r[]
end

"""
    solve(dm::DeviceMatrix, b; rtol=1e-10, maxit=20000, mode=GT_SOLVE_FP64) -> x, SolveInfo
"""
function solve(dm::DeviceMatrix, b::Vector{Float64}; rtol=1e-10, maxit=20000, mode=GT_SOLVE_FP64)
    x = zeros(Float64, length(b))
    info = Ref(SolveInfo(0, 0, 0.0, 0, 0))
    check(dm.space.ctx.h, ccall((:gt_solve, LIB), Cint,
                                (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Float64, Cint, Cint, Ref{SolveInfo}),
                                dm.h, b, x, rtol, maxit, mode, info))
    x, info[]
end

end # module
