"""
    KagomeVMC

Carlo.jl plugin for KagomeDSL.jl that runs the Monte Carlo hot path on a
GB300 through libkvmc (the C ABI of include/kvmc.h).  It drops in for the
reference's `MC` type and its callbacks (src/MonteCarlo.jl:165, :435, :538,
:628, :675, :715, :751): the mean-field set-up stays in KagomeDSL
(`DoubleKagome`, `Hamiltonian`), the orbitals and bonds go to the GPU, and
every walker of a batch is one independent chain there.

One `Carlo.sweep!` call runs `proposals_per_sweep` exchange proposals per
walker in one library call (default min(N_up, N_down), the reference's
refresh and measurement interval), with the local energy sampled inside the
call at the reference's cadence; `Carlo.measure!` pushes the batch mean of
those samples as `:OL`.  `proposals_per_sweep = 1` gives one proposal per
`sweep!` call as in the reference, at one library call per proposal.

Indices cross the boundary 0-based; configuration values keep the
reference's meaning (0 empty, 1..n label).  The library path defaults to
the in-tree build and can be overridden with the KVMC_LIBRARY environment
variable.
"""
module KagomeVMC

using Carlo
using HDF5
using KagomeDSL
using LinearAlgebra

export MC

const libkvmc = get(ENV, "KVMC_LIBRARY", joinpath(@__DIR__, "..", "kagomedsl.jl_gb300", "_build", "libkvmc.so"))

# enum values of include/kvmc.h
const KVMC_OK = Int32(0)
const KVMC_ERR_ARGUMENT = Int32(1)
const KVMC_ERR_BOUNDS = Int32(2)
const KVMC_ERR_SINGULAR = Int32(3)
const KVMC_PLAIN_FP64 = Int32(0)
const KVMC_MIXED_FP32 = Int32(1)
const KVMC_ACCEPT_REFERENCE = Int32(0)
const KVMC_ACCEPT_METROPOLIS = Int32(1)
const KVMC_W_AUTO = Int32(0)
const KVMC_W_HBM = Int32(2)
const KVMC_TUNE_WARP_WALKERS = Int32(5)
const KVMC_TUNE_COND_HI = Int32(6)
const KVMC_TUNE_COND_LO = Int32(7)
const KVMC_TUNE_REFRESH32 = Int32(4)
const KVMC_TUNE_DRIFT_SEVERE = Int32(9)
const KVMC_TUNE_CLUSTER = Int32(10)

# the C structs, field for field (kvmc_lattice_desc, kvmc_link, kvmc_model_desc,
# kvmc_batch_desc, kvmc_sweep_stats)
struct LatticeDesc
    n1::Int32
    n2::Int32
    pbc::NTuple{2,Int32}
    antipbc::NTuple{2,Int32}
    t::Float64
end

struct Link
    label1::Int32
    label2::Int32
    dx::Int32
    dy::Int32
    amplitude::Float64
end

struct ModelDesc
    n_sites::Int32
    n_up::Int32
    n_down::Int32
    n_bonds::Int32
    bonds::Ptr{Int32}
    U_up::Ptr{Float64}
    U_down::Ptr{Float64}
    U_up_imag::Ptr{Float64}
    U_down_imag::Ptr{Float64}
end

struct BatchDesc
    n_walkers::Int32
    precision::Int32
    accept_rule::Int32
    refresh_interval::Int32
    measure_interval::Int32
    delay_k::Int32
    device::Int32
    seed::UInt64
    w_placement::Int32
end

struct SweepStats
    proposals::Int64
    accepted::Int64
    measurements::Int64
    sum_energy::Float64
    sum_energy2::Float64
    refreshes::Int64
    max_drift::Float64
    bad_walkers::Int32
    launches::Int32
    fp64_redos::Int64
end

SweepStats() = SweepStats(0, 0, 0, 0.0, 0.0, 0, 0.0, 0, 0)

"""Maps a libkvmc status onto the reference's exceptions (include/kvmc.h)."""
function check(rc::Integer, h::Ptr{Cvoid} = C_NULL)
    rc == KVMC_OK && return nothing
    buf = zeros(UInt8, 1024)
    ccall((:kvmc_last_error, libkvmc), Cint, (Ptr{Cvoid}, Ptr{UInt8}, Csize_t), h, buf, length(buf))
    msg = GC.@preserve buf unsafe_string(pointer(buf))
    rc == KVMC_ERR_ARGUMENT && throw(ArgumentError(msg))
    rc == KVMC_ERR_BOUNDS && throw(BoundsError(msg))
    rc == KVMC_ERR_SINGULAR && error("QR-based configuration is singular. The Hamiltonian may be rank-deficient.")
    error("libkvmc: " * msg)
end

# --- thin wrappers, one per entry point ---------------------------------------

kvmc_version() = (abi = Ref{Int32}(0); arch = Ref{Int32}(0);
    check(ccall((:kvmc_version, libkvmc), Cint, (Ref{Int32}, Ref{Int32}), abi, arch)); (abi[], arch[]))

function kvmc_create(md::ModelDesc, bd::BatchDesc)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:kvmc_create, libkvmc), Cint, (Ref{ModelDesc}, Ref{BatchDesc}, Ref{Ptr{Cvoid}}), md, bd, h))
    return h[]
end

kvmc_destroy(h::Ptr{Cvoid}) = ccall((:kvmc_destroy, libkvmc), Cint, (Ptr{Cvoid},), h)

kvmc_init(h, ku, kd) = check(ccall((:kvmc_init, libkvmc), Cint, (Ptr{Cvoid}, Ptr{Int32}, Ptr{Int32}, Ptr{Int32}),
                                   h, ku, kd, C_NULL), h)

function kvmc_sweep(h, proposals::Integer)
    st = Ref(SweepStats())
    check(ccall((:kvmc_sweep, libkvmc), Cint, (Ptr{Cvoid}, Int64, Ref{SweepStats}), h, proposals, st), h)
    return st[]
end

function kvmc_advance(h, moves::Integer)
    st = Ref(SweepStats())
    check(ccall((:kvmc_advance, libkvmc), Cint, (Ptr{Cvoid}, Int64, Ref{SweepStats}), h, moves, st), h)
    return st[]
end

kvmc_measure(h, e::Vector{Float64}) = check(ccall((:kvmc_measure, libkvmc), Cint, (Ptr{Cvoid}, Ptr{Float64}), h, e), h)

kvmc_get_state(h, ku, kd, ct) = check(ccall((:kvmc_get_state, libkvmc), Cint,
    (Ptr{Cvoid}, Ptr{Int32}, Ptr{Int32}, Ptr{Int64}), h, ku, kd, ct), h)

kvmc_set_state(h, ku, kd, ct) = check(ccall((:kvmc_set_state, libkvmc), Cint,
    (Ptr{Cvoid}, Ptr{Int32}, Ptr{Int32}, Ptr{Int64}), h, ku, kd, ct), h)

kvmc_set_tuning(h, key::Int32, value::Integer) = check(ccall((:kvmc_set_tuning, libkvmc), Cint,
    (Ptr{Cvoid}, Int32, Int32), h, key, value), h)

kvmc_refresh(h) = check(ccall((:kvmc_refresh, libkvmc), Cint, (Ptr{Cvoid},), h), h)

kvmc_walker_stats(h, se, se2, nm, acc, prop, status) = check(ccall((:kvmc_walker_stats, libkvmc), Cint,
    (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Int64}, Ptr{Int64}, Ptr{Int64}, Ptr{Int32}),
    h, se, se2, nm, acc, prop, status), h)

function kvmc_hopping_matrix(lat::LatticeDesc, B::Real)
    ns = Ref{Int32}(0)
    check(ccall((:kvmc_lattice_sites, libkvmc), Cint, (Ref{LatticeDesc}, Ref{Int32}), lat, ns))
    H = zeros(Float64, 2 * ns[] * ns[])
    check(ccall((:kvmc_hopping_matrix, libkvmc), Cint,
        (Ref{LatticeDesc}, Ptr{Link}, Int32, Ptr{Link}, Int32, Float64, Ptr{Float64}),
        lat, C_NULL, 0, C_NULL, 0, B, H))
    Hc = reshape(H, 2, ns[], ns[])
    return complex.(Hc[1, :, :], Hc[2, :, :])
end

# --- the reference's start for one walker -------------------------------------

"""
Pivoted-QR start restated from src/MonteCarlo.jl:326-357: the columns of
U_up^T picked by a pivoted QR are the up sites, then the down sites are
picked the same way among the remaining sites (N_down = ns - N_up as at
:339).  Returns 0/label configuration vectors.
"""
function qr_start(U_up::AbstractMatrix, U_down::AbstractMatrix, ns::Integer, N_up::Integer)
    p_up = qr(transpose(U_up), ColumnNorm()).p
    up = p_up[1:N_up]
    ku = zeros(Int32, ns)
    ku[up] .= 1:N_up
    kd = zeros(Int32, ns)
    rest = setdiff(1:ns, up)
    N_down = ns - N_up
    if N_down > 0
        p_dn = qr(transpose(U_down[rest, :]), ColumnNorm()).p
        kd[rest[p_dn[1:N_down]]] .= 1:N_down
    end
    return ku, kd
end

# --- the Carlo.jl plugin -------------------------------------------------------

mutable struct MC <: AbstractMC
    Ham::KagomeDSL.Hamiltonian
    h::Ptr{Cvoid}
    walkers::Int
    ns::Int
    proposals_per_sweep::Int
    last::SweepStats          # the statistics of the last sweep! call
    keep::Vector{Any}         # host arrays the handle was created from
end

"""
    MC(params)

`params` holds the reference's keys (:n1, :n2, :PBC, :antiPBC, :lattice,
:B, :N_up, :N_down) plus :walkers (default 1), :precision (:mixed or
:plain, default :mixed), :accept (:reference or :metropolis),
:refresh_interval, :delay_k, :warp_walkers (one warp per walker, this many
per CTA; 0 = one CTA per walker), :proposals_per_sweep, :seed and :device.
"""
function MC(params::AbstractDict)
    lattice = get(params, :lattice, DoubleKagome)
    lat = lattice(1.0, params[:n1], params[:n2], params[:PBC]; antiPBC = get(params, :antiPBC, (false, false)))
    Ham = KagomeDSL.Hamiltonian(params[:N_up], params[:N_down], lat; B = get(params, :B, 0.0))
    ns = size(Ham.U_up, 1)
    bonds = Int32[x - 1 for b in Ham.nn for x in b]                 # 0-based (i, j) pairs
    Uu = Matrix{Float64}(real(Ham.U_up))
    Ud = Matrix{Float64}(real(Ham.U_down))
    cplx = any(!iszero, imag(Ham.U_up)) || any(!iszero, imag(Ham.U_down))
    Uui = Matrix{Float64}(imag(Ham.U_up))
    Udi = Matrix{Float64}(imag(Ham.U_down))
    walkers = get(params, :walkers, 1)
    precision = get(params, :precision, :mixed) == :plain ? KVMC_PLAIN_FP64 : KVMC_MIXED_FP32
    accept = get(params, :accept, :reference) == :metropolis ? KVMC_ACCEPT_METROPOLIS : KVMC_ACCEPT_REFERENCE
    warp = get(params, :warp_walkers, 0)
    h = GC.@preserve bonds Uu Ud Uui Udi begin
        md = ModelDesc(ns, size(Uu, 2), size(Ud, 2), length(Ham.nn), pointer(bonds), pointer(Uu), pointer(Ud),
                       cplx ? pointer(Uui) : C_NULL, cplx ? pointer(Udi) : C_NULL)
        bd = BatchDesc(walkers, precision, accept, get(params, :refresh_interval, 0), 0, get(params, :delay_k, 0),
                       get(params, :device, 0), get(params, :seed, 0), warp > 0 ? KVMC_W_HBM : KVMC_W_AUTO)
        kvmc_create(md, bd)
    end
    nocc = min(params[:N_up], params[:N_down])
    mc = MC(Ham, h, walkers, ns, get(params, :proposals_per_sweep, nocc), SweepStats(), Any[bonds, Uu, Ud, Uui, Udi])
    finalizer(m -> (m.h != C_NULL && kvmc_destroy(m.h); m.h = C_NULL), mc)
    if warp > 0
        kvmc_set_tuning(h, KVMC_TUNE_WARP_WALKERS, warp)
        kvmc_set_tuning(h, KVMC_TUNE_COND_HI, get(params, :guard_hi, 200))
        kvmc_set_tuning(h, KVMC_TUNE_COND_LO, get(params, :guard_lo, 20))
    end
    return mc
end

"""Carlo.init! (src/MonteCarlo.jl:435-441): the reference's QR start for one
walker, seeded random starts (redrawn until tilde_U is regular) for a batch."""
function Carlo.init!(mc::MC, ctx::MCContext, params::AbstractDict)
    if mc.walkers == 1 && get(params, :init, :qr) == :qr
        ku, kd = qr_start(real(mc.Ham.U_up), real(mc.Ham.U_down), mc.ns, params[:N_up])
        kvmc_init(mc.h, ku, kd)
    else
        kvmc_init(mc.h, C_NULL, C_NULL)
    end
    return nothing
end

"""Carlo.sweep! (src/MonteCarlo.jl:538-607): proposals_per_sweep proposals per
walker in one call; records the batch acceptance fraction as :acc."""
function Carlo.sweep!(mc::MC, ctx::MCContext)
    mc.last = kvmc_sweep(mc.h, mc.proposals_per_sweep)
    measure!(ctx, :acc, mc.last.accepted / max(mc.last.proposals, 1))
    return nothing
end

"""Carlo.measure! (src/MonteCarlo.jl:628-634): the batch mean of the local
energies the last sweep! sampled at the reference's cadence; with fewer
proposals per sweep than that cadence, a measurement of the current state
when the cadence is due."""
function Carlo.measure!(mc::MC, ctx::MCContext)
    if mc.last.measurements > 0
        measure!(ctx, :OL, mc.last.sum_energy / mc.last.measurements)
    elseif (ctx.sweeps * mc.proposals_per_sweep) % min(mc.Ham.N_up, mc.Ham.N_down) == 0
        e = zeros(Float64, mc.walkers)
        kvmc_measure(mc.h, e)
        measure!(ctx, :OL, sum(e) / length(e))
    end
    return nothing
end

"""Carlo.register_evaluables (src/MonteCarlo.jl:675-687): energy = OL / ns."""
function Carlo.register_evaluables(::Type{MC}, eval::Evaluator, params::AbstractDict)
    ns = params[:n1] * params[:n2] * 3
    evaluate!(eval, :energy, (:OL,)) do OL
        return OL / ns
    end
    return nothing
end

"""Carlo.write_checkpoint (src/MonteCarlo.jl:715-719): configurations per walker
(an ns x walkers matrix: the C layout [walker][site]) and the position in
each walker's proposal stream."""
function Carlo.write_checkpoint(mc::MC, out::HDF5.Group)
    ku = zeros(Int32, mc.ns, mc.walkers)
    kd = similar(ku)
    ct = zeros(Int64, mc.walkers)
    kvmc_get_state(mc.h, ku, kd, ct)
    out["kappa_up"] = Int.(ku)
    out["kappa_down"] = Int.(kd)
    out["counters"] = ct
    return nothing
end

"""Carlo.read_checkpoint! (src/MonteCarlo.jl:751-755): W is rebuilt on the
device from the restored configurations."""
function Carlo.read_checkpoint!(mc::MC, in::HDF5.Group)
    ku = Int32.(read(in, "kappa_up"))
    kd = Int32.(read(in, "kappa_down"))
    ct = haskey(in, "counters") ? Int64.(read(in, "counters")) : C_NULL
    kvmc_set_state(mc.h, ku, kd, ct)
    return nothing
end

end # module
