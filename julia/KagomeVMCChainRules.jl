"""
    KagomeVMCChainRules

The adjoint energy gradient of libkvmc as a ChainRulesCore `rrule`:
`vmc_energy(α)` samples E(α) for the extended ansatz α = (t2, m, θ)
(include/kvmc.h, kvmc_ansatz_hopping) on the GPU, and its pullback returns
ΔE · ∂E/∂α from the same samples (kvmc_set_log_derivatives,
kvmc_measure_grad, kvmc_grad_sums).  No reference counterpart: the reference
evaluates the energy of the π-flux state only.

The orbital derivatives come from first-order perturbation of the host
diagonalisation that builds the orbitals:
    dU[:, c] = Σ_{m unoccupied} v_m (v_mᴴ dH v_c) / (ε_c − ε_m)
(occupied–occupied mixing multiplies every determinant by one constant and
is dropped).  The estimate follows include/kvmc.h:
    ∂E/∂α_a = 2 Re(⟨conj(O_a) E_L⟩ − conj(⟨O_a⟩) ⟨E_L⟩)
with the per-walker weighted sums of kvmc_grad_sums.
"""
module KagomeVMCChainRules

using ChainRulesCore
using LinearAlgebra

include(joinpath(@__DIR__, "KagomeVMC.jl"))
using .KagomeVMC: libkvmc, check, LatticeDesc, Link, ModelDesc, BatchDesc, kvmc_create, kvmc_destroy,
                  kvmc_init, kvmc_sweep, KVMC_MIXED_FP32, KVMC_ACCEPT_REFERENCE, KVMC_W_AUTO

export vmc_energy

const NPARAMS = 3

function ansatz(lat::LatticeDesc, α::AbstractVector{Float64}; B = 0.0)
    ns = Ref{Int32}(0)
    check(ccall((:kvmc_lattice_sites, libkvmc), Cint, (Ref{LatticeDesc}, Ref{Int32}), lat, ns))
    N = Int(ns[])
    H = zeros(Float64, 2 * N * N)
    dH = zeros(Float64, 2 * NPARAMS * N * N)
    params = collect(Float64, α)
    check(ccall((:kvmc_ansatz_hopping, libkvmc), Cint,
        (Ref{LatticeDesc}, Ptr{Link}, Int32, Ptr{Link}, Int32, Float64, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
        lat, C_NULL, 0, C_NULL, 0, B, params, H, dH))
    Hc = reshape(H, 2, N, N)
    dHc = reshape(dH, 2, N, N, NPARAMS)
    return complex.(Hc[1, :, :], Hc[2, :, :]), [complex.(dHc[1, :, :, a], dHc[2, :, :, a]) for a in 1:NPARAMS]
end

"""The nearest-neighbour bonds of the α = 0 hopping matrix, 0-based."""
function bonds(lat::LatticeDesc; B = 0.0)
    H0, _ = ansatz(lat, zeros(NPARAMS); B = B)
    N = size(H0, 1)
    Hflat = zeros(Float64, 2 * N * N)
    Hflat[1:2:end] .= vec(real(H0))
    Hflat[2:2:end] .= vec(imag(H0))
    nb = Ref{Int32}(0)
    check(ccall((:kvmc_bonds_from_hopping, libkvmc), Cint, (Int32, Ptr{Float64}, Ref{Int32}, Ptr{Int32}),
                N, Hflat, nb, C_NULL))
    out = zeros(Int32, 2 * nb[])
    check(ccall((:kvmc_bonds_from_hopping, libkvmc), Cint, (Int32, Ptr{Float64}, Ref{Int32}, Ptr{Int32}),
                N, Hflat, nb, out))
    return out
end

function orbitals_and_derivatives(H, dHs, n)
    F = eigen(Hermitian(H))
    ε, V = F.values, F.vectors
    U = V[:, 1:n]
    occ, emp = 1:n, n+1:size(H, 1)
    ε[n+1] - ε[n] > 1e-10 || throw(ArgumentError("no gap at the Fermi level: the orbital derivatives are undefined"))
    dUs = map(dHs) do dH
        M = V[:, emp]' * dH * V[:, occ]                      # (unoccupied, occupied)
        V[:, emp] * (M ./ (ε[occ]' .- ε[emp]))
    end
    return U, dUs
end

struct Estimate
    E::Float64
    grad::Vector{Float64}
end

"""dE/dα from the per-walker sums (layout of kvmc_grad_sums, include/kvmc.h)."""
function estimate(sums::Matrix{Float64}, P::Int)
    t = vec(sum(sums; dims = 2))                            # sums[:, walker] summed over walkers
    w = t[1]
    E = complex(t[2], t[3]) / w
    O = [complex(t[4 + 2a], t[5 + 2a]) / w for a in 0:P-1]
    OE = [complex(t[4 + 2P + 2a], t[5 + 2P + 2a]) / w for a in 0:P-1]
    grad = [2 * real(OE[a] - conj(O[a]) * E) for a in 1:P]
    return Estimate(real(E), grad)
end

"""
    vmc_energy(α; n1, n2, N_up, N_down, walkers = 1024, sweeps = 100, thermalize = 20, seed = 1)

E(α) per site, sampled with `walkers` chains of the mixed form, one adjoint
evaluation after each n-proposal sweep.
"""
vmc_energy(α::AbstractVector{Float64}; kw...) = first(energy_and_gradient(α; kw...))

function energy_and_gradient(α::AbstractVector{Float64}; n1, n2, N_up, N_down, walkers = 1024, sweeps = 100,
                             thermalize = 20, seed = 1, B = 0.0)
    lat = LatticeDesc(n1, n2, (1, 1), (0, 1), 1.0)
    H, dHs = ansatz(lat, α; B = B)
    N = size(H, 1)
    n = min(N_up, N_down)
    Uu, dUu = orbitals_and_derivatives(H, dHs, N_up)
    Ud, dUd = orbitals_and_derivatives(H, dHs, N_down)
    bd_ = bonds(lat; B = B)
    re(x) = Matrix{Float64}(real(x))
    im_(x) = Matrix{Float64}(imag(x))
    keep = (re(Uu), im_(Uu), re(Ud), im_(Ud))
    h = GC.@preserve bd_ keep begin
        md = ModelDesc(N, N_up, N_down, length(bd_) ÷ 2, pointer(bd_), pointer(keep[1]), pointer(keep[3]),
                       pointer(keep[2]), pointer(keep[4]))
        kvmc_create(md, BatchDesc(walkers, KVMC_MIXED_FP32, KVMC_ACCEPT_REFERENCE, 0, 0, 0, 0, seed, KVMC_W_AUTO))
    end
    try
        # [P] column-major N x n matrices per spin, real and imaginary parts apart
        dur = reduce(hcat, re.(dUu)); dui = reduce(hcat, im_.(dUu))
        ddr = reduce(hcat, re.(dUd)); ddi = reduce(hcat, im_.(dUd))
        check(ccall((:kvmc_set_log_derivatives, libkvmc), Cint,
            (Ptr{Cvoid}, Int32, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
            h, NPARAMS, dur, dui, ddr, ddi), h)
        kvmc_init(h, C_NULL, C_NULL)
        kvmc_sweep(h, thermalize * n)
        check(ccall((:kvmc_reset_stats, libkvmc), Cint, (Ptr{Cvoid},), h), h)
        for _ in 1:sweeps
            kvmc_sweep(h, n)
            check(ccall((:kvmc_measure_grad, libkvmc), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}),
                        h, C_NULL, C_NULL), h)
        end
        L = 3 + 4 * NPARAMS + 2 * NPARAMS^2
        sums = zeros(Float64, L, walkers)
        check(ccall((:kvmc_grad_sums, libkvmc), Cint, (Ptr{Cvoid}, Ptr{Float64}), h, sums), h)
        est = estimate(sums, NPARAMS)
        return est.E / N, est.grad ./ N
    finally
        kvmc_destroy(h)
    end
end

function ChainRulesCore.rrule(::typeof(vmc_energy), α::AbstractVector{Float64}; kw...)
    E, g = energy_and_gradient(α; kw...)
    vmc_energy_pullback(ΔE) = (NoTangent(), ΔE .* g)
    return E, vmc_energy_pullback
end

end # module
