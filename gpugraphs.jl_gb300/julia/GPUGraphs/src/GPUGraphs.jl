"""
    GPUGraphs

Drop-in replacement of GPUGraphs.jl's module (src/GPUGraphs.jl:1-53) backed by
libgpugraphs.so, the hand-written sm_103a kernels, through `ccall`.  Same exported
names, keyword arguments, 1-based indices and exceptions; device arrays are
CUDA.jl `CuArray`s.  There is no KernelAbstractions backend and no CPU fallback:
operators must be GPUGraphs_* functions (or the Base functions mapped below).

Set ENV["GPUGRAPHS_LIB"] to the library path, or keep the default
(`../../lib/libgpugraphs.so` relative to this file).
"""
module GPUGraphs

using CUDA
using SparseArrays
using LinearAlgebra

const LIB = get(ENV, "GPUGRAPHS_LIB",
                joinpath(@__DIR__, "..", "..", "..", "lib", "libgpugraphs.so"))

export AbstractSparseGPUMatrix, SparseGPUMatrixCSR, SparseGPUMatrixSELL, gpu_spmv!, gpu_spmm!,
       sprand_gpu, monoid_neutral, monoid_absorb, bfs_distances, bfs_distances!, bfs_parents,
       bfs_parents!, shortest_path, shortest_path!, GPUGraphs_add, GPUGraphs_safe_add,
       GPUGraphs_mul, GPUGraphs_second, GPUGraphs_band, GPUGraphs_bor, GPUGraphs_any,
       GPUGraphs_secondi, GPUGraphs_max, GPUGraphs_min, SparseGPUVector, AbstractSparseGPUVector,
       SparseGPUMatrixCSC,
       gpu_spmspv!, gpu_spmspv, gpu_spmv_rows!, gpu_ewise!, gpu_apply!, gpu_reduce, read_rb,
       read_mtx, read_edgelist

# ---------------------------------------------------------------------------------
# algebra (src/algebra.jl): same functions, plus their operator codes in the C ABI
# ---------------------------------------------------------------------------------
monoid_neutral(type::Type, op::Function) =
    error("monoid_neutral not implemented for type $(type) and operation $(op)")
monoid_absorb(type::Any, op::Any) = nothing

GPUGraphs_first(x, _, _, _, _, _) = x
GPUGraphs_second(_, y, _, _, _, _) = y
GPUGraphs_any(x, y, _, _, _, _) = max(x, y)
GPUGraphs_pair(x, y, _, _, _, _) = ifelse(y != zero(y), one(x), zero(x))
GPUGraphs_add(x, y, _, _, _, _) = x + y
GPUGraphs_safe_add(x, y, _, _, _, _) =
    ifelse(max(x, y) == max(typemax(x), typemax(y)), max(typemax(x), typemax(y)), x + y)
GPUGraphs_minus(x, y, _, _, _, _) = x - y
GPUGraphs_rminus(x, y, _, _, _, _) = y - x
GPUGraphs_mul(x, y, _, _, _, _) = x * y
GPUGraphs_min(x, y, _, _, _, _) = min(x, y)
GPUGraphs_max(x, y, _, _, _, _) = max(x, y)
GPUGraphs_lor(x, y, _, _, _, _) = x | y
GPUGraphs_land(x, y, _, _, _, _) = x & y
GPUGraphs_bor(x, y, _, _, _, _) = x | y
GPUGraphs_band(x, y, _, _, _, _) = x & y
GPUGraphs_bxor(x, y, _, _, _, _) = x ⊻ y
GPUGraphs_firsti(_, _, A_i, _, _, _) = A_i
GPUGraphs_firstj(_, _, _, A_j, _, _) = A_j
GPUGraphs_secondi(_, y, _, _, B_i, _) = B_i * y
GPUGraphs_secondj(_, _, _, _, _, B_j) = B_j

monoid_neutral(::Type{T}, ::typeof(GPUGraphs_any)) where {T} = zero(T)
monoid_absorb(::Type{T}, ::typeof(GPUGraphs_any)) where {T} = Any
monoid_neutral(::Type{T}, ::typeof(GPUGraphs_add)) where {T} = zero(T)
monoid_absorb(::Type{T}, ::typeof(GPUGraphs_add)) where {T} = typemax(T)
monoid_neutral(::Type{T}, ::typeof(GPUGraphs_safe_add)) where {T} = zero(T)
monoid_absorb(::Type{T}, ::typeof(GPUGraphs_safe_add)) where {T} = typemax(T)
monoid_neutral(::Type{T}, ::typeof(GPUGraphs_mul)) where {T} = one(T)
monoid_absorb(::Type{T}, ::typeof(GPUGraphs_mul)) where {T} = zero(T)
monoid_neutral(::Type{T}, ::typeof(GPUGraphs_min)) where {T} = typemax(T)
monoid_absorb(::Type{T}, ::typeof(GPUGraphs_min)) where {T} = typemin(T)
monoid_neutral(::Type{T}, ::typeof(GPUGraphs_max)) where {T} = typemin(T)
monoid_absorb(::Type{T}, ::typeof(GPUGraphs_max)) where {T} = typemax(T)
monoid_neutral(::Type{Bool}, ::typeof(GPUGraphs_lor)) = false
monoid_absorb(::Type{Bool}, ::typeof(GPUGraphs_lor)) = true
monoid_neutral(::Type{Bool}, ::typeof(GPUGraphs_land)) = true
monoid_absorb(::Type{Bool}, ::typeof(GPUGraphs_land)) = false
monoid_neutral(::Type{T}, ::typeof(GPUGraphs_bor)) where {T} = zero(T)
monoid_absorb(::Type{T}, ::typeof(GPUGraphs_bor)) where {T} = ~zero(T)
monoid_neutral(::Type{T}, ::typeof(GPUGraphs_band)) where {T} = ~zero(T)
monoid_absorb(::Type{T}, ::typeof(GPUGraphs_band)) where {T} = zero(T)

const OPCODE = IdDict{Any,Cint}(
    GPUGraphs_first => 1, GPUGraphs_second => 2, GPUGraphs_any => 3, GPUGraphs_pair => 4,
    GPUGraphs_add => 5, GPUGraphs_safe_add => 6, GPUGraphs_minus => 7, GPUGraphs_rminus => 8,
    GPUGraphs_mul => 9, GPUGraphs_min => 10, GPUGraphs_max => 11, GPUGraphs_lor => 12,
    GPUGraphs_land => 13, GPUGraphs_bor => 14, GPUGraphs_band => 15, GPUGraphs_bxor => 16,
    GPUGraphs_firsti => 17, GPUGraphs_firstj => 18, GPUGraphs_secondi => 19,
    GPUGraphs_secondj => 20,
    (+) => 5, (*) => 9, min => 10, max => 11, (|) => 14, (&) => 15)

opcode(f) = haskey(OPCODE, f) ? OPCODE[f] :
    throw(ArgumentError("operator $(f) has no sm_103a kernel; use a GPUGraphs_* operator"))

dtcode(::Type{Bool}) = Cint(1)
dtcode(::Type{Int32}) = Cint(2)
dtcode(::Type{Int64}) = Cint(3)
dtcode(::Type{Float32}) = Cint(4)
dtcode(::Type{Float64}) = Cint(5)
dtcode(::Type{T}) where {T} = throw(ArgumentError("element type $(T) is not supported"))

# ---------------------------------------------------------------------------------
# status codes -> Julia exceptions
# ---------------------------------------------------------------------------------
lasterror() = unsafe_string(ccall((:gg_last_error, LIB), Cstring, ()))

function check(rc::Cint)
    rc == 0 && return nothing
    msg = lasterror()
    rc == 1 && throw(DimensionMismatch(msg))
    (rc == 2 || rc == 3) && throw(ArgumentError(msg))
    rc == 4 && throw(MethodError(msg, ()))
    rc == 5 && throw(OutOfMemoryError())
    rc == 8 && throw(BoundsError(msg))
    rc == 9 && throw(AssertionError(msg))
    error("libgpugraphs error $(rc): $(msg)")
end

const CTX = Dict{Int,Ptr{Cvoid}}()

function ctx()
    dev = CUDA.deviceid(CUDA.device())
    c = get!(CTX, dev) do
        r = Ref{Ptr{Cvoid}}(C_NULL)
        check(ccall((:gg_init, LIB), Cint, (Cint, Ptr{Ptr{Cvoid}}), dev, r))
        r[]
    end
    # work goes on the task's CUDA.jl stream, ordered with the caller's own kernels
    check(ccall((:gg_set_stream, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}), c,
                CUDA.stream().handle))
    return c
end

# ---------------------------------------------------------------------------------
# storage (src/storage/*.jl)
# ---------------------------------------------------------------------------------
abstract type AbstractSparseGPUMatrix{Tv,Ti<:Integer} <: SparseArrays.AbstractSparseMatrix{Tv,Ti} end

mutable struct SparseGPUMatrixCSR{Tv,Ti<:Integer} <: AbstractSparseGPUMatrix{Tv,Ti}
    handle::Ptr{Cvoid}
    m::Int
    n::Int
    rowptr::CuArray{Ti,1}
    colval::CuArray{Ti,1}
    nzval::CuArray{Tv,1}
end

mutable struct SparseGPUMatrixSELL{Tv,Ti<:Integer} <: AbstractSparseGPUMatrix{Tv,Ti}
    handle::Ptr{Cvoid}
    m::Int
    n::Int
    perm::Vector{Int}
    slice_size::Int
    nslices::Int
    nnz::Int
    n_stored::Int
    slice_ptr::CuArray{Ti,1}
    colval::CuArray{Ti,1}
    nzval::CuArray{Tv,1}
end

function _finalize!(A)
    A.handle == C_NULL && return
    ccall((:gg_mat_destroy, LIB), Cint, (Ptr{Cvoid},), A.handle)
    A.handle = C_NULL
end

function _arrays(h, ::Type{Tv}, lens) where {Tv}
    p = Ref{Ptr{Cvoid}}(); c = Ref{Ptr{Cvoid}}(); v = Ref{Ptr{Cvoid}}(); q = Ref{Ptr{Cvoid}}()
    check(ccall((:gg_mat_arrays, LIB), Cint,
                (Ptr{Cvoid}, Ptr{Ptr{Cvoid}}, Ptr{Ptr{Cvoid}}, Ptr{Ptr{Cvoid}}, Ptr{Ptr{Cvoid}}),
                h, p, c, v, q))
    wrap(ptr, T, len) = unsafe_wrap(CuArray, CuPtr{T}(UInt(ptr)), len; own = false)
    return wrap(p[], Int32, lens[1]), wrap(c[], Int32, lens[2]), wrap(v[], Tv, lens[3]),
           wrap(q[], Int32, lens[4])
end

"""
    SparseGPUMatrixCSR(m, n, rowptr, colval, nzval[, backend])

src/storage/CSR.jl:34-92: 1-based CSR on the device, validated by the library
(ArgumentError on bad lengths, rowptr ends or out-of-range columns).
"""
function SparseGPUMatrixCSR(m::Int, n::Int, rowptr::AbstractVector, colval::AbstractVector,
                            nzval::AbstractVector{Tv}, backend = nothing) where {Tv}
    length(rowptr) != m + 1 && throw(ArgumentError("length(rowptr) must be equal to m + 1"))
    length(colval) != length(nzval) &&
        throw(ArgumentError("length(colval) must be equal to length(nzval)"))
    rp = Vector{Int32}(Array(rowptr)); cv = Vector{Int32}(Array(colval)); nz = Vector{Tv}(Array(nzval))
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:gg_csr_create, LIB), Cint,
                (Ptr{Cvoid}, Int64, Int64, Int64, Ptr{Int32}, Ptr{Int32}, Ptr{Cvoid}, Cint, Cint,
                 Ptr{Ptr{Cvoid}}), ctx(), m, n, length(cv), rp, cv, nz, dtcode(Tv), 0, h))
    r, c, v, _ = _arrays(h[], Tv, (m + 1, length(cv), length(cv), 0))
    A = SparseGPUMatrixCSR{Tv,Int32}(h[], m, n, r, c, v)
    finalizer(_finalize!, A)
    return A
end

# CSR.jl:95-104: CSR of a transposed CSC without copying its structure
SparseGPUMatrixCSR(m::Transpose{Tv,<:SparseMatrixCSC{Tv}}, backend = nothing) where {Tv} =
    SparseGPUMatrixCSR(size(m.parent, 2), size(m.parent, 1), m.parent.colptr, m.parent.rowval,
                       m.parent.nzval)
SparseGPUMatrixCSR(m::Matrix{Tv}, backend = nothing) where {Tv} =
    SparseGPUMatrixCSR(transpose(sparse(transpose(m))))
SparseGPUMatrixCSR(m::SparseMatrixCSC{Tv}, backend = nothing) where {Tv} =
    SparseGPUMatrixCSR(transpose(sparse(transpose(m))))
SparseGPUMatrixCSR(::Type{Tv}, ::Type{Ti}, backend = nothing) where {Tv,Ti} =
    SparseGPUMatrixCSR(0, 0, ones(Int32, 1), Int32[], Tv[])
SparseGPUMatrixCSR(m::Int, n::Int, ::Type{Tv}, ::Type{Ti}, backend = nothing) where {Tv,Ti} =
    SparseGPUMatrixCSR(m, n, ones(Int32, m + 1), Int32[], Tv[])

"""
    SparseGPUMatrixSELL(A, [backend,] slice_size = 32; sigma = 1)

src/storage/SELL.jl:99-181 built on the device; sigma > 1 sorts rows by length
within windows of sigma rows (SELL-C-sigma).
"""
function SparseGPUMatrixSELL(A::SparseGPUMatrixCSR{Tv}, slice_size::Int = 32; sigma::Int = 1) where {Tv}
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:gg_sell_create, LIB), Cint, (Ptr{Cvoid}, Ptr{Cvoid}, Int64, Int64, Ptr{Ptr{Cvoid}}),
                ctx(), A.handle, slice_size, sigma, h))
    info = [Ref{Int64}() for _ in 1:6]
    fmt = Ref{Cint}(); dt = Ref{Cint}()
    check(ccall((:gg_mat_info, LIB), Cint,
                (Ptr{Cvoid}, Ptr{Cint}, Ptr{Int64}, Ptr{Int64}, Ptr{Int64}, Ptr{Cint}, Ptr{Int64},
                 Ptr{Int64}, Ptr{Int64}), h[], fmt, info[1], info[2], info[3], dt, info[4], info[5], info[6]))
    m, n, nz, nst, C, ns = (x[] for x in info)
    sp, cv, v, pm = _arrays(h[], Tv, (ns + 1, nst, nst, m))
    S = SparseGPUMatrixSELL{Tv,Int32}(h[], m, n, Vector{Int}(Array(pm)), C, ns, nz, nst, sp, cv, v)
    finalizer(_finalize!, S)
    return S
end
SparseGPUMatrixSELL(m, backend, slice_size::Int = 32; sigma::Int = 1) =
    SparseGPUMatrixSELL(SparseGPUMatrixCSR(m), slice_size; sigma = sigma)

Base.size(A::AbstractSparseGPUMatrix) = (A.m, A.n)
Base.size(A::AbstractSparseGPUMatrix, i::Int) = (i == 1) ? A.m : A.n
Base.length(A::AbstractSparseGPUMatrix) = A.m * A.n
SparseArrays.nnz(A::SparseGPUMatrixCSR) = length(A.nzval)
SparseArrays.nnz(A::SparseGPUMatrixSELL) = A.nnz

sprand_gpu(::Type{Tv}, m::Int, n::Int, p::Real, backend = nothing) where {Tv} =
    SparseGPUMatrixCSR(transpose(SparseArrays.sprand(Tv, m, n, p)))

# ---------------------------------------------------------------------------------
# kernels (src/spmv/*.jl, src/spmm/*.jl)
# ---------------------------------------------------------------------------------
function gpu_spmv!(C::CuVector{Tr}, A::AbstractSparseGPUMatrix{Tv}, B::CuVector{Tx};
                   mul::Function = GPUGraphs_mul, add::Function = GPUGraphs_add,
                   accum::Function = GPUGraphs_second,
                   range::Union{Nothing,UnitRange} = nothing,
                   mask::Union{Nothing,AbstractVector} = nothing) where {Tr,Tv,Tx}
    size(A, 2) != length(B) && throw(DimensionMismatch("Matrix dimensions must agree"))
    size(C, 1) != size(A, 1) && throw(DimensionMismatch("Matrix dimensions must agree"))
    promote_type(Tv, Tx) <: Tr ||
        throw(ArgumentError("Result type must be able to hold the result of the multiplication"))
    mp, mt, ml = C_NULL, Cint(0), Int64(0)
    if mask !== nothing
        length(mask) != size(A, 1) &&
            throw(DimensionMismatch("Mask length must be equal to the number of rows in A"))
        mp, mt, ml = pointer(mask), dtcode(eltype(mask)), length(mask)
    end
    lo, hi = range === nothing ? (0, 0) : (first(range), last(range))
    check(ccall((:gg_spmv, LIB), Cint,
                (Ptr{Cvoid}, Ptr{Cvoid}, Cint, Cint, Cint, CuPtr{Cvoid}, Cint, Int64, CuPtr{Cvoid},
                 Cint, Int64, CuPtr{Cvoid}, Cint, Int64, Int64, Int64),
                ctx(), A.handle, opcode(mul), opcode(add), opcode(accum), pointer(C), dtcode(Tr),
                length(C), pointer(B), dtcode(Tx), length(B), mp, mt, ml, lo, hi))
    return nothing
end

function gpu_spmm!(C::CuMatrix{Tr}, A::AbstractSparseGPUMatrix{Tv}, B::CuMatrix{Tx};
                   mul::Function = GPUGraphs_mul, add::Function = GPUGraphs_add,
                   accum::Function = GPUGraphs_second,
                   mask::Union{Nothing,AbstractVector} = nothing,
                   range::Union{Nothing,UnitRange{Int}} = nothing) where {Tr,Tv,Tx}
    @assert size(A, 2) == size(B, 1)
    @assert size(C, 1) == size(A, 1)
    @assert size(C, 2) == size(B, 2)
    mp, mt, ml = C_NULL, Cint(0), Int64(0)
    if mask !== nothing
        mp, mt, ml = pointer(mask), dtcode(eltype(mask)), length(mask)
    end
    lo, hi = range === nothing ? (0, 0) : (first(range), last(range))
    check(ccall((:gg_spmm, LIB), Cint,
                (Ptr{Cvoid}, Ptr{Cvoid}, Cint, Cint, Cint, CuPtr{Cvoid}, Cint, Int64, Int64,
                 CuPtr{Cvoid}, Cint, Int64, Int64, Int64, Cint, CuPtr{Cvoid}, Cint, Int64, Int64, Int64),
                ctx(), A.handle, opcode(mul), opcode(add), opcode(accum), pointer(C), dtcode(Tr),
                size(C, 1), size(C, 1), pointer(B), dtcode(Tx), size(B, 1), size(B, 1), size(B, 2),
                Cint(0), mp, mt, ml, lo, hi))
    return nothing
end

# ---------------------------------------------------------------------------------
# algorithms (src/algorithms/*.jl)
# ---------------------------------------------------------------------------------
function bfs_distances!(A_T::AbstractSparseGPUMatrix, source::Integer, dist::CuVector{Int32},
                        curr = nothing, next = nothing, to_explore = nothing)
    lv = Ref{Int64}(0)
    check(ccall((:gg_bfs_levels, LIB), Cint,
                (Ptr{Cvoid}, Ptr{Cvoid}, Int64, CuPtr{Int32}, Int64, Ptr{Int64}),
                ctx(), A_T.handle, source, pointer(dist), length(dist), lv))
    return nothing
end

function bfs_distances(A_T::AbstractSparseGPUMatrix, source::Integer; use_mask = true)
    dist = CUDA.fill(typemax(Int32), size(A_T, 1))
    bfs_distances!(A_T, source, dist)
    return dist
end

function bfs_parents!(A_T::AbstractSparseGPUMatrix, source::Integer, parents::CuVector{Int32},
                      curr = nothing, next = nothing, to_explore = nothing, batch_size::Int = 8)
    lv = Ref{Int64}(0)
    check(ccall((:gg_bfs_parents, LIB), Cint,
                (Ptr{Cvoid}, Ptr{Cvoid}, Int64, CuPtr{Int32}, Int64, Cint, Ptr{Int64}),
                ctx(), A_T.handle, source, pointer(parents), length(parents), Cint(0), lv))
    return nothing
end

function bfs_parents(A_T::AbstractSparseGPUMatrix, source::Integer; batch_size::Int = 8)
    parents = CUDA.fill(typemax(Int32), size(A_T, 1))
    bfs_parents!(A_T, source, parents)
    return parents
end

_tdist(::AbstractSparseGPUMatrix{Tv}) where {Tv} = Tv == Bool ? Int32 : Tv

function _sssp!(A_T, sources::Vector{Int64}, dist, next)
    r = Ref{Int64}(0)
    check(ccall((:gg_sssp, LIB), Cint,
                (Ptr{Cvoid}, Ptr{Cvoid}, Ptr{Int64}, Int64, CuPtr{Cvoid}, CuPtr{Cvoid}, Cint, Int64,
                 Ptr{Int64}), ctx(), A_T.handle, sources, length(sources), pointer(dist),
                next === nothing ? CuPtr{Cvoid}(0) : pointer(next), dtcode(eltype(dist)),
                size(A_T, 1), r))
    return nothing
end

function shortest_path(A_T::AbstractSparseGPUMatrix, source::Integer)
    dist = CuVector{_tdist(A_T)}(undef, size(A_T, 1))
    _sssp!(A_T, Int64[source], dist, nothing)
    return dist
end

function shortest_path(A_T::AbstractSparseGPUMatrix, sources::AbstractVector{<:Integer})
    dist = CuMatrix{_tdist(A_T)}(undef, size(A_T, 1), length(sources))
    _sssp!(A_T, Vector{Int64}(sources), dist, nothing)
    return dist
end

shortest_path!(A_T::AbstractSparseGPUMatrix, source::Integer, dist, next, updated = nothing,
               diff = nothing) = _sssp!(A_T, Int64[source], dist, next)
shortest_path!(A_T::AbstractSparseGPUMatrix, sources::AbstractVector{<:Integer}, dist, next,
               updated = nothing, diff = nothing) = _sssp!(A_T, Vector{Int64}(sources), dist, next)

# ---------------------------------------------------------------------------------
# sparse vectors (src/GPUGraphsVector.jl), SpMSpV (src/spmspv.jl), the sparse-mask
# kernel (src/spmv/CSR.jl:90-115), CSC SpMV (src/spmv/CSC.jl) and the e-wise /
# map-reduce steps the reference leaves to broadcasts
# ---------------------------------------------------------------------------------
abstract type AbstractSparseGPUVector{Tv,Ti<:Integer} <: SparseArrays.AbstractSparseVector{Tv,Ti} end

mutable struct SparseGPUVector{Tv,Ti<:Integer} <: AbstractSparseGPUVector{Tv,Ti}
    n::Int
    nzind::CuVector{Ti}
    nzval::CuVector{Tv}
end

function SparseGPUVector(n::Integer, nzind::AbstractVector, nzval::AbstractVector{Tv},
                         backend = nothing) where {Tv}
    length(nzind) != length(nzval) &&
        throw(ArgumentError("length(nzind) must be equal to length(nzval)"))
    return SparseGPUVector{Tv,Int32}(Int(n), CuVector{Int32}(nzind), CuVector{Tv}(nzval))
end
SparseGPUVector(v::SparseVector{Tv}, backend = nothing) where {Tv} =
    SparseGPUVector(length(v), v.nzind, v.nzval)
function SparseGPUVector(v::Vector{Tv}, backend = nothing) where {Tv}
    nzind = findall(!iszero, v)
    return SparseGPUVector(length(v), nzind, v[nzind])
end
Base.size(V::AbstractSparseGPUVector) = (V.n,)
Base.length(V::AbstractSparseGPUVector) = V.n
SparseArrays.nnz(V::AbstractSparseGPUVector) = length(V.nzval)
SparseArrays.nonzeroinds(V::AbstractSparseGPUVector) = V.nzind
SparseArrays.nonzeros(V::AbstractSparseGPUVector) = V.nzval

"""
    gpu_spmspv!(C, A, B::SparseGPUVector; mul, add, accum) -> rows

For every row i of A holding an entry whose column carries an entry of B,
C[i] = accum(C[i], add over those entries of mul(A[i, j], B[j], i, j, j, 1)) in storage
order; returns the 1-based rows written, ascending.
"""
function gpu_spmspv!(C::CuVector{Tr}, A::SparseGPUMatrixCSR{Tv}, B::SparseGPUVector{Tx};
                     mul::Function = GPUGraphs_mul, add::Function = GPUGraphs_add,
                     accum::Function = GPUGraphs_second) where {Tr,Tv,Tx}
    size(A, 2) != B.n && throw(DimensionMismatch("Matrix dimensions must agree"))
    size(C, 1) != size(A, 1) && throw(DimensionMismatch("Matrix dimensions must agree"))
    rows = CuVector{Int32}(undef, max(size(A, 1), 1))
    cnt = Ref{Int64}(0)
    check(ccall((:gg_spmspv, LIB), Cint,
                (Ptr{Cvoid}, Ptr{Cvoid}, Cint, Cint, Cint, CuPtr{Cvoid}, Cint, Int64, CuPtr{Int32},
                 CuPtr{Cvoid}, Cint, Int64, Int64, CuPtr{Int32}, Ptr{Int64}),
                ctx(), A.handle, opcode(mul), opcode(add), opcode(accum), pointer(C), dtcode(Tr),
                length(C), pointer(B.nzind), pointer(B.nzval), dtcode(Tx), length(B.nzind), B.n,
                pointer(rows), cnt))
    return rows[1:cnt[]]
end

function gpu_spmspv(A::SparseGPUMatrixCSR{Tv}, B::SparseGPUVector{Tx};
                    mul::Function = GPUGraphs_mul, add::Function = GPUGraphs_add) where {Tv,Tx}
    C = CUDA.zeros(promote_type(Tv, Tx), size(A, 1))
    rows = gpu_spmspv!(C, A, B; mul = mul, add = add, accum = GPUGraphs_second)
    return SparseGPUVector{eltype(C),Int32}(size(A, 1), rows, C[rows])
end

function gpu_spmv_rows!(C::CuVector{Tr}, A::SparseGPUMatrixCSR{Tv}, B::CuVector{Tx},
                        rows::CuVector{Int32}; mul::Function = GPUGraphs_mul,
                        add::Function = GPUGraphs_add,
                        accum::Function = GPUGraphs_second) where {Tr,Tv,Tx}
    check(ccall((:gg_spmv_rows, LIB), Cint,
                (Ptr{Cvoid}, Ptr{Cvoid}, Cint, Cint, Cint, CuPtr{Cvoid}, Cint, Int64, CuPtr{Cvoid},
                 Cint, Int64, CuPtr{Int32}, Int64),
                ctx(), A.handle, opcode(mul), opcode(add), opcode(accum), pointer(C), dtcode(Tr),
                length(C), pointer(B), dtcode(Tx), length(B), pointer(rows), length(rows)))
    return nothing
end

# CSC: held as the CSR storage of the transpose (same colptr / rowval / nzval)
mutable struct SparseGPUMatrixCSC{Tv,Ti<:Integer} <: AbstractSparseGPUMatrix{Tv,Ti}
    t::SparseGPUMatrixCSR{Tv,Ti}
    m::Int
    n::Int
    colptr::CuVector{Ti}
    rowval::CuVector{Ti}
    nzval::CuVector{Tv}
end

function SparseGPUMatrixCSC(m::Int, n::Int, colptr::AbstractVector, rowval::AbstractVector,
                            nzval::AbstractVector{Tv}, backend = nothing) where {Tv}
    t = SparseGPUMatrixCSR(n, m, colptr, rowval, nzval)
    return SparseGPUMatrixCSC{Tv,Int32}(t, m, n, t.rowptr, t.colval, t.nzval)
end
SparseGPUMatrixCSC(A::SparseMatrixCSC{Tv}, backend = nothing) where {Tv} =
    SparseGPUMatrixCSC(size(A, 1), size(A, 2), A.colptr, A.rowval, A.nzval)

function gpu_spmv!(C::CuVector{Tr}, A::SparseGPUMatrixCSC{Tv}, B::CuVector{Tx};
                   mul::Function = GPUGraphs_mul, add::Function = GPUGraphs_add,
                   accum::Function = GPUGraphs_second,
                   range::Union{Nothing,UnitRange} = nothing,
                   mask::Union{Nothing,AbstractVector} = nothing) where {Tr,Tv,Tx}
    size(A, 2) != length(B) && throw(DimensionMismatch("Matrix dimensions must agree"))
    size(C, 1) != size(A, 1) && throw(DimensionMismatch("Matrix dimensions must agree"))
    mp, mt, ml = mask === nothing ? (C_NULL, Cint(0), Int64(0)) :
                 (pointer(mask), dtcode(eltype(mask)), Int64(length(mask)))
    lo, hi = range === nothing ? (0, 0) : (first(range), last(range))
    check(ccall((:gg_spmv_t, LIB), Cint,
                (Ptr{Cvoid}, Ptr{Cvoid}, Cint, Cint, Cint, CuPtr{Cvoid}, Cint, Int64, CuPtr{Cvoid},
                 Cint, Int64, CuPtr{Cvoid}, Cint, Int64, Int64, Int64),
                ctx(), A.t.handle, opcode(mul), opcode(add), opcode(accum), pointer(C), dtcode(Tr),
                length(C), pointer(B), dtcode(Tx), length(B), mp, mt, ml, lo, hi))
    return nothing
end

function gpu_ewise!(z::CuVector{Tz}, x::CuVector{Tx}, y::CuVector{Ty}, op::Function;
                    mask::Union{Nothing,CuVector} = nothing) where {Tz,Tx,Ty}
    check(ccall((:gg_ewise, LIB), Cint,
                (Ptr{Cvoid}, Cint, CuPtr{Cvoid}, Cint, CuPtr{Cvoid}, Cint, CuPtr{Cvoid}, Cint, Int64,
                 CuPtr{Cvoid}, Cint),
                ctx(), opcode(op), pointer(z), dtcode(Tz), pointer(x), dtcode(Tx), pointer(y),
                dtcode(Ty), length(z), mask === nothing ? CU_NULL : pointer(mask),
                mask === nothing ? Cint(0) : dtcode(eltype(mask))))
    return z
end

function gpu_apply!(z::CuVector{Tz}, x::CuVector{Tx}, s::Ts, op::Function;
                    bind_first::Bool = false, mask::Union{Nothing,CuVector} = nothing) where {Tz,Tx,Ts}
    sr = Ref{Ts}(s)
    check(ccall((:gg_apply, LIB), Cint,
                (Ptr{Cvoid}, Cint, CuPtr{Cvoid}, Cint, CuPtr{Cvoid}, Cint, Ptr{Cvoid}, Cint, Cint,
                 Int64, CuPtr{Cvoid}, Cint),
                ctx(), opcode(op), pointer(z), dtcode(Tz), pointer(x), dtcode(Tx), sr, dtcode(Ts),
                Cint(bind_first), length(z), mask === nothing ? CU_NULL : pointer(mask),
                mask === nothing ? Cint(0) : dtcode(eltype(mask))))
    return z
end

function gpu_reduce(x::CuVector{T}, add::Function) where {T}
    out = Ref{T}()
    check(ccall((:gg_reduce, LIB), Cint, (Ptr{Cvoid}, Cint, CuPtr{Cvoid}, Cint, Int64, Ptr{Cvoid}),
                ctx(), opcode(add), pointer(x), dtcode(T), length(x), out))
    return out[]
end

# graph files (host): Rutherford-Boeing / Harwell-Boeing matrices and edge lists
function _take_host(cp, rv, vv, ncol, nnz)
    colptr = copy(unsafe_wrap(Array, Ptr{Int32}(cp[]), ncol + 1))
    rowval = copy(unsafe_wrap(Array, Ptr{Int32}(rv[]), nnz))
    vals = copy(unsafe_wrap(Array, Ptr{Float64}(vv[]), nnz))
    for p in (cp[], rv[], vv[])
        ccall((:gg_host_free, LIB), Cint, (Ptr{Cvoid},), p)
    end
    return colptr, rowval, vals
end

function read_rb(path::AbstractString; expand_symmetric::Bool = true)
    m = Ref{Int64}(); n = Ref{Int64}(); nnz = Ref{Int64}(); kind = Ref{Cint}()
    cp = Ref{Ptr{Cvoid}}(); rv = Ref{Ptr{Cvoid}}(); vv = Ref{Ptr{Cvoid}}()
    check(ccall((:gg_read_rb, LIB), Cint,
                (Cstring, Cint, Ptr{Int64}, Ptr{Int64}, Ptr{Int64}, Ptr{Ptr{Cvoid}}, Ptr{Ptr{Cvoid}},
                 Ptr{Ptr{Cvoid}}, Ptr{Cint}), path, Cint(expand_symmetric), m, n, nnz, cp, rv, vv, kind))
    colptr, rowval, vals = _take_host(cp, rv, vv, n[], nnz[])
    return SparseMatrixCSC{Float64,Int32}(m[], n[], colptr, rowval, vals)
end

function read_mtx(path::AbstractString; expand_symmetric::Bool = true)
    m = Ref{Int64}(); n = Ref{Int64}(); nnz = Ref{Int64}(); kind = Ref{Cint}()
    cp = Ref{Ptr{Cvoid}}(); rv = Ref{Ptr{Cvoid}}(); vv = Ref{Ptr{Cvoid}}()
    check(ccall((:gg_read_mtx, LIB), Cint,
                (Cstring, Cint, Ptr{Int64}, Ptr{Int64}, Ptr{Int64}, Ptr{Ptr{Cvoid}}, Ptr{Ptr{Cvoid}},
                 Ptr{Ptr{Cvoid}}, Ptr{Cint}), path, Cint(expand_symmetric), m, n, nnz, cp, rv, vv, kind))
    colptr, rowval, vals = _take_host(cp, rv, vv, n[], nnz[])
    return SparseMatrixCSC{Float64,Int32}(m[], n[], colptr, rowval, vals)
end

# adjacency A (A[u, v] for the edge u -> v) of an edge-list file
function read_edgelist(path::AbstractString; base::Integer = 1)
    nv = Ref{Int64}(); nnz = Ref{Int64}(); w = Ref{Cint}()
    cp = Ref{Ptr{Cvoid}}(); rv = Ref{Ptr{Cvoid}}(); vv = Ref{Ptr{Cvoid}}()
    check(ccall((:gg_read_edgelist, LIB), Cint,
                (Cstring, Cint, Ptr{Int64}, Ptr{Int64}, Ptr{Ptr{Cvoid}}, Ptr{Ptr{Cvoid}},
                 Ptr{Ptr{Cvoid}}, Ptr{Cint}), path, Cint(base), nv, nnz, cp, rv, vv, w))
    colptr, rowval, vals = _take_host(cp, rv, vv, nv[], nnz[])
    return SparseMatrixCSC{Float64,Int32}(nv[], nv[], colptr, rowval, vals)
end

end # module
