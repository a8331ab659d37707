# ------------------------------------------------------------------
# GeoStatsProcessesGPU — GPUSEQSIM, sequential Gaussian simulation on one
# GB300, plugged into GeoStatsProcesses.jl's field-simulation method API
# through libgeosgs.so (include/geosgs.h).
#
#   using GeoStatsProcesses, GeoStatsProcessesGPU
#   ens = rand(rng, GaussianProcess(γ), grid, 256; data,
#              method=GPUSEQSIM(path=RandomPath(), maxneighbors=48))
#
# GPUSEQSIM plugs in the way SEQSIM does (src/simulation/field/seqsim.jl:42-156):
# a FieldSimulationMethod subtype (src/simulation/field.jl:135) with
# `preprocess` and `randsingle` methods; `rand` (src/simulation/field.jl:73-124)
# is not overridden.  The path is drawn once in `preprocess` and shared by all
# realizations of the call; `randsingle` simulates realizations in blocks of
# `batch` on the GPU and hands them out one by one.
# ------------------------------------------------------------------
module GeoStatsProcessesGPU

using Random
using LinearAlgebra: I
using Distributed: myid
using Meshes
using GeoTables
using GeoStatsFunctions
using Unitful: ustrip
using Distances: Euclidean
using GeoStatsProcesses
import GeoStatsProcesses: preprocess, randsingle, FieldSimulationMethod

export GPUSEQSIM

const libgeosgs = get(ENV, "GEOSGS_LIB",
  joinpath(@__DIR__, "..", "geosgs", "lib", "libgeosgs.so"))

# ---- C structs (field order and types of include/geosgs.h) ----
struct SgsVariogram
  type::Int32
  reserved::Int32
  sill::Float64
  nugget::Float64
  ranges::NTuple{3,Float64}
  rotation::NTuple{9,Float64}
end

struct SgsBall
  radii::NTuple{3,Float64}
  rotation::NTuple{9,Float64}
end

struct SgsProblem
  dim::Int32
  dims::NTuple{3,Int32}
  origin::NTuple{3,Float64}
  spacing::NTuple{3,Float64}
  ndata::Int64
  data_coords::Ptr{Float64}
  data_values::Ptr{Float64}
  variogram::SgsVariogram
  mean::Float64
  minneighbors::Int32
  maxneighbors::Int32
  search::Int32
  precision::Int32
  ball::SgsBall
  path::Ptr{Int32}
  refine_steps::Int32
  warm_start::Int32
  device::Int32
  flags::Int32
  nstructures::Int32
  reserved2::Int32
  structures::Ptr{SgsVariogram}
end

const SGS_SEARCH_RANGE, SGS_SEARCH_BALL, SGS_SEARCH_NEAREST = Int32(0), Int32(1), Int32(2)

"""
    GPUSEQSIM(; path, minneighbors, maxneighbors, neighborhood, distance, precision, refine_steps, batch, device)

SEQSIM's options (`path`, `minneighbors`, `maxneighbors`, `neighborhood`,
`distance`; seqsim.jl:42-48, same defaults) plus `precision` (`:fp32` = FP32
solves with FP64 refinement, `:fp64`), `refine_steps`, `batch`
(realizations simulated per GPU call) and `device`.  `distance` must be the
Euclidean distance (the GPU search computes Euclidean and ellipsoid metrics
only); anything else is an `ArgumentError`.
"""
Base.@kwdef struct GPUSEQSIM{P,N,D} <: FieldSimulationMethod
  path::P = LinearPath()
  minneighbors::Int = 1
  maxneighbors::Int = 26
  neighborhood::N = :range
  distance::D = Euclidean()
  precision::Symbol = :fp32
  refine_steps::Int = 2
  batch::Int = 64
  device::Int = 0
end

mutable struct GPUPlan
  ptr::Ptr{Cvoid}
  owner::Int
  function GPUPlan(ptr)
    p = new(ptr, myid())
    finalizer(p) do q
      q.ptr == C_NULL || ccall((:sgs_plan_destroy, libgeosgs), Cvoid, (Ptr{Cvoid},), q.ptr)
      q.ptr = C_NULL
    end
  end
end

function check(rc, ptr)
  rc == 0 && return
  msg = unsafe_string(ccall((:sgs_last_error, libgeosgs), Cstring, (Ptr{Cvoid},), ptr))
  rc == -1 ? throw(ArgumentError(msg)) : error("libgeosgs ($rc): $msg")
end

vtype(::SphericalVariogram) = Int32(1)
vtype(::ExponentialVariogram) = Int32(2)
vtype(::GaussianVariogram) = Int32(3)
vtype(f) = throw(ArgumentError("GPUSEQSIM supports spherical, exponential and gaussian variograms and their sums"))

# the structures of a (nested) model: a NestedVariogram c1 g1 + c2 g2 + ...
# gives structure i the sill c_i sill(g_i) and nugget c_i nugget(g_i)
structures(f::NestedVariogram) = [(Float64(c), g) for (c, g) in zip(f.cs, f.γs)]
structures(f) = [(1.0, f)]

pad3(t, fill) = ntuple(i -> i <= length(t) ? Float64(t[i]) : fill, 3)
# radii of a ball; a 1D problem runs as the n x 1 grid, whose second axis
# then takes the same radius (every lag's second component is 0)
radii3(b, dim) = dim == 1 ? (Float64(ustrip(first(radii(b)))), Float64(ustrip(first(radii(b)))), 1.0) :
                            pad3(ustrip.(radii(b)), 1.0)

function rot9(R, dim)
  M = Matrix{Float64}(I(3))
  M[1:dim, 1:dim] .= Matrix(R)[1:dim, 1:dim]
  ntuple(k -> M[(k - 1) % 3 + 1, (k - 1) ÷ 3 + 1], 9)  # column-major, leading dimension 3
end

# Geometry, neighbourhood, data and path of a problem -> a created plan; the
# `before_prepare` hook runs between sgs_plan_create and sgs_plan_prepare.
function _plan(vgs::Vector{SgsVariogram}, mean, method::GPUSEQSIM, grid, data, datavals; before_prepare=identity)
  grid isa CartesianGrid || throw(ArgumentError("GPUSEQSIM simulates on a CartesianGrid"))
  method.distance isa Euclidean || throw(ArgumentError("GPUSEQSIM supports the Euclidean distance only"))
  1 <= length(vgs) <= 4 || throw(ArgumentError("GPUSEQSIM takes 1 to 4 nested structures"))
  vg, more = vgs[1], vgs[2:end]
  dim = embeddim(grid)
  cdim = dim == 1 ? 2 : dim  # 1D: the n x 1 grid with the data on the row's centre line (y = 0.5)
  dims = size(grid)
  orig = ustrip.(to(minimum(grid)))
  spac = ustrip.(spacing(grid))
  nb = method.neighborhood
  search, sball = if nb === :range
    SGS_SEARCH_RANGE, SgsBall((1.0, 1.0, 1.0), rot9(I(3), dim))
  elseif nb isa MetricBall
    SGS_SEARCH_BALL, SgsBall(radii3(nb, dim), rot9(rotation(nb), dim))
  else
    SGS_SEARCH_NEAREST, SgsBall((1.0, 1.0, 1.0), rot9(I(3), dim))
  end
  # data appended after the grid nodes, as SEQSIM's ExplicitInit (seqsim.jl:211-218,267-271)
  xy = Float64[]
  vals = Float64.(datavals)
  if !isnothing(data)
    for i in 1:nrow(data)
      c = ustrip.(to(centroid(GeoTables.domain(data), i)))
      append!(xy, dim == 1 ? (c[1], 0.5) : c)
    end
  end
  path = Int32.(collect(traverse(grid, method.path)) .- 1)  # one path for all realizations
  planref = Ref{Ptr{Cvoid}}(C_NULL)
  GC.@preserve xy vals path more begin
    prob = SgsProblem(Int32(cdim), pad3(dims, 1.0) .|> Int32, pad3(orig, 0.0), pad3(spac, 1.0),
                      length(vals), pointer(xy), pointer(vals), vg, Float64(mean),
                      method.minneighbors, method.maxneighbors, search,
                      method.precision === :fp64 ? Int32(0) : Int32(1), sball, pointer(path),
                      method.refine_steps, 0, method.device, 0,
                      length(more), 0, isempty(more) ? Ptr{SgsVariogram}(C_NULL) : pointer(more))
    check(ccall((:sgs_plan_create, libgeosgs), Cint, (Ref{SgsProblem}, Ref{Ptr{Cvoid}}), prob, planref), C_NULL)
  end
  plan = GPUPlan(planref[])
  before_prepare(plan)
  check(ccall((:sgs_plan_prepare, libgeosgs), Cint, (Ptr{Cvoid},), plan.ptr), plan.ptr)
  plan
end

function preprocess(rng::AbstractRNG, process::GaussianProcess, method::GPUSEQSIM, init, domain, data)
  f = process.func
  nvariables(f) > 1 && return _preprocess_multivariate(process, method, domain, data)
  dim = embeddim(domain)
  vgs = [SgsVariogram(vtype(g), 0, c * ustrip(sill(g)), c * ustrip(nugget(g)), radii3(g.ball, dim),
                      rot9(rotation(g.ball), dim)) for (c, g) in structures(f)]
  var = isnothing(data) ? :field : first(propertynames(values(data)))
  vals = isnothing(data) ? Float64[] : Float64.(ustrip.(getproperty(values(data), var)))
  plan = _plan(vgs, ustrip(process.mean), method, domain, data, vals)
  (; plan, var, nelm=nelements(domain), block=Ref(Matrix{Float64}(undef, 0, 0)), cursor=Ref(0))
end

function randsingle(rng::AbstractRNG, process::GaussianProcess, method::GPUSEQSIM, domain, data, preproc)
  hasproperty(preproc, :vars) && return _randsingle_multivariate(rng, method, preproc)
  (; plan, var, nelm, block, cursor) = preproc
  # the plan lives on this process's GPU (src/simulation/field.jl:98-100 style check)
  myid() == plan.owner || throw(ArgumentError("GPUSEQSIM realizations must run on the process that prepared them"))
  if cursor[] == size(block[], 2)
    B = Matrix{Float64}(undef, nelm, method.batch)  # N x batch, column = realization
    check(ccall((:sgs_plan_simulate, libgeosgs), Cint,
                (Ptr{Cvoid}, Int32, Ptr{Float64}, UInt64, Ptr{Float64}),
                plan.ptr, method.batch, C_NULL, rand(rng, UInt64), B), plan.ptr)
    block[] = B
    cursor[] = 0
  end
  cursor[] += 1
  (; var => block[][:, cursor[]])
end

# ---- sequential indicator simulation (seqsim.jl:247-261, 292-310, 342-347) ----
# For proportional transiograms t_ab(h) = p_b + (delta_ab - p_b) rho(h) every
# category's simple cokriging weights are rho's simple kriging weights, so the
# plan solves with rho (the transiogram's family, its range, sill 1, nugget 0)
# and sgs_plan_simulate_indicator draws the categories.
ctype(::SphericalTransiogram) = Int32(1)
ctype(::ExponentialTransiogram) = Int32(2)
ctype(::GaussianTransiogram) = Int32(3)
ctype(f) = throw(ArgumentError("GPUSEQSIM simulates proportional spherical, exponential and gaussian transiograms"))

# A multivariate covariance A_1 * C_1 + A_2 * C_2 + ... (GeoStatsFunctions'
# NestedCovariance with matrix coefficients, nvariables(f) = L) is a linear
# model of coregionalization: each node solves the full simple cokriging
# system (sgs_plan_set_indicator_cokriging), the structures C_s passed as
# the problem's nested variogram and the A_s as the coregionalization matrices.
vtype(::SphericalCovariance) = Int32(1)
vtype(::ExponentialCovariance) = Int32(2)
vtype(::GaussianCovariance) = Int32(3)

function _lmc(f::NestedCovariance, dim)
  vgs = [SgsVariogram(vtype(g), 0, ustrip(sill(g)), ustrip(nugget(g)), radii3(g.ball, dim),
                      rot9(rotation(g.ball), dim)) for g in f.fs]
  coef = Float64[]
  for A in f.cs
    M = Matrix{Float64}(A isa Number ? fill(A, 1, 1) : A)
    append!(coef, vec(permutedims(M)))  # row-major, as the C side reads it
  end
  vgs, coef
end

function preprocess(rng::AbstractRNG, process::IndicatorProcess, method::GPUSEQSIM, init, domain, data)
  f = process.func
  prob = Float64.(collect(process.prob))
  2 <= length(prob) <= 8 || throw(ArgumentError("GPUSEQSIM simulates 2 to 8 categories"))
  f isa NestedCovariance && return _preprocess_cokriging(process, method, domain, data, prob)
  r = Float64(ustrip(range(f)))
  rho = SgsVariogram(ctype(f), 0, 1.0, 0.0, (r, r, r), rot9(I(3), embeddim(domain)))
  # categories: the data's sorted distinct labels (the one-hot transform), 1..L without data
  var = isnothing(data) ? :field : first(propertynames(values(data)))
  labels = isnothing(data) ? collect(1:length(prob)) : sort(unique(getproperty(values(data), var)))
  isnothing(data) || length(labels) == length(prob) ||
    throw(ArgumentError("probabilities must have $(length(labels)) components, received $(length(prob))"))
  cats = isnothing(data) ? Int32[] : Int32.(indexin(getproperty(values(data), var), labels) .- 1)
  setind(plan) = GC.@preserve prob cats check(ccall((:sgs_plan_set_indicator, libgeosgs), Cint,
                                                     (Ptr{Cvoid}, Int32, Ptr{Float64}, Ptr{Int32}),
                                                     plan.ptr, length(prob), prob, cats), plan.ptr)
  plan = _plan([rho], 0.0, method, domain, data, zeros(length(cats)); before_prepare=setind)
  (; plan, var, labels, nelm=nelements(domain), block=Ref(Matrix{Int32}(undef, 0, 0)), cursor=Ref(0))
end

function _preprocess_cokriging(process, method, domain, data, prob)
  vgs, coef = _lmc(process.func, embeddim(domain))
  length(coef) == length(vgs) * length(prob)^2 ||
    throw(ArgumentError("coregionalization matrices must be $(length(prob)) x $(length(prob))"))
  var = isnothing(data) ? :field : first(propertynames(values(data)))
  labels = isnothing(data) ? collect(1:length(prob)) : sort(unique(getproperty(values(data), var)))
  isnothing(data) || length(labels) == length(prob) ||
    throw(ArgumentError("probabilities must have $(length(labels)) components, received $(length(prob))"))
  cats = isnothing(data) ? Int32[] : Int32.(indexin(getproperty(values(data), var), labels) .- 1)
  setcok(plan) = GC.@preserve prob cats coef check(ccall((:sgs_plan_set_indicator_cokriging, libgeosgs), Cint,
                                                         (Ptr{Cvoid}, Int32, Ptr{Float64}, Ptr{Int32}, Ptr{Float64}),
                                                         plan.ptr, length(prob), prob, cats, coef), plan.ptr)
  plan = _plan(vgs, 0.0, method, domain, data, zeros(length(cats)); before_prepare=setcok)
  (; plan, var, labels, nelm=nelements(domain), block=Ref(Matrix{Int32}(undef, 0, 0)), cursor=Ref(0))
end

function randsingle(rng::AbstractRNG, process::IndicatorProcess, method::GPUSEQSIM, domain, data, preproc)
  (; plan, var, labels, nelm, block, cursor) = preproc
  myid() == plan.owner || throw(ArgumentError("GPUSEQSIM realizations must run on the process that prepared them"))
  if cursor[] == size(block[], 2)
    B = Matrix{Int32}(undef, nelm, method.batch)  # N x batch, column = realization
    check(ccall((:sgs_plan_simulate_indicator, libgeosgs), Cint,
                (Ptr{Cvoid}, Int32, Ptr{Float64}, UInt64, Ptr{Int32}),
                plan.ptr, method.batch, C_NULL, rand(rng, UInt64), B), plan.ptr)
    block[] = B
    cursor[] = 0
  end
  cursor[] += 1
  (; var => labels[block[][:, cursor[]] .+ 1])
end

# ---- multivariate Gaussian simulation (gaussian.jl:22-35; seqsim.jl:277-290,
# 302-304, 335-340) ----
# A GaussianProcess whose func is a linear model of coregionalization (a
# NestedCovariance with matrix coefficients, nvariables(f) = L > 1): each node
# solves the simple cokriging system of its neighbours' L values and draws all
# L variables at once from the conditional MvNormal (sgs_plan_set_multivariate,
# sgs_plan_simulate_multivariate).  Every datum holds all L variables.
function _preprocess_multivariate(process, method, domain, data)
  f = process.func
  f isa NestedCovariance || throw(ArgumentError("GPUSEQSIM simulates multivariate processes of a linear model of coregionalization"))
  L = nvariables(f)
  L <= 8 || throw(ArgumentError("GPUSEQSIM simulates up to 8 variables"))
  vgs, coef = _lmc(f, embeddim(domain))
  length(coef) == length(vgs) * L^2 || throw(ArgumentError("coregionalization matrices must be $L x $L"))
  mean = Float64.(ustrip.(collect(process.mean)))
  vars = isnothing(data) ? ntuple(i -> Symbol(:field, i), L) : Tuple(propertynames(values(data)))
  length(vars) == L || throw(ArgumentError("the data must have $L variables, one per variable of the process"))
  D = isnothing(data) ? 0 : nrow(data)
  dv = Float64[]  # D x L, row-major
  for i in 1:D, v in vars
    push!(dv, Float64(ustrip(getproperty(values(data), v)[i])))
  end
  setmv(plan) = GC.@preserve mean coef dv check(ccall((:sgs_plan_set_multivariate, libgeosgs), Cint,
                                                      (Ptr{Cvoid}, Int32, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
                                                      plan.ptr, L, mean, coef, dv), plan.ptr)
  plan = _plan(vgs, 0.0, method, domain, data, zeros(D); before_prepare=setmv)
  (; plan, vars, L, nelm=nelements(domain), block=Ref(Array{Float64,3}(undef, 0, 0, 0)), cursor=Ref(0))
end

function _randsingle_multivariate(rng, method, preproc)
  (; plan, vars, L, nelm, block, cursor) = preproc
  myid() == plan.owner || throw(ArgumentError("GPUSEQSIM realizations must run on the process that prepared them"))
  if cursor[] == size(block[], 3)
    B = Array{Float64,3}(undef, nelm, L, method.batch)  # N x L x batch: the C side's nreals x L x N
    check(ccall((:sgs_plan_simulate_multivariate, libgeosgs), Cint,
                (Ptr{Cvoid}, Int32, Ptr{Float64}, UInt64, Ptr{Float64}),
                plan.ptr, method.batch, C_NULL, rand(rng, UInt64), B), plan.ptr)
    block[] = B
    cursor[] = 0
  end
  cursor[] += 1
  NamedTuple{vars}(Tuple(block[][:, a, cursor[]] for a in 1:L))
end

end # module
