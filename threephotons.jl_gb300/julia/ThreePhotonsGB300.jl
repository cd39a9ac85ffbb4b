# ThreePhotonsGB300 -- binds libtp3 (include/tp3.h) behind ThreePhotons.jl's own calls.
#
# Written against the reference's Julia 0.6 API (src/correlations.jl, src/cuda.jl,
# src/determination.jl).  Not run in this build: neither the build machine nor the GPU
# machine has Julia.  The same C ABI is exercised from Python by the test suite.
#
# Use inside a session that has loaded ThreePhotons:
#     include("ThreePhotonsGB300.jl"); using ThreePhotonsGB300
#     ThreePhotons.complexBasis_choice = ThreePhotonsGB300.GB300_calculate_basis
# after which rotate_all_at_once / calculate_temperature / evaluate_step call
# FullCorrelation_parallized and energy on a BasisTypeGB300 (methods below).
module ThreePhotonsGB300

import ThreePhotons: AbstractBasisType, SphericalHarmonicsVolume, FullCorrelation_parallized, energy,
                     Umat, C3, num_coeff, loadPDB, atomfactorlist

export BasisTypeGB300, GB300_calculate_basis, GB300_chains_create, GB300_chains_run, GB300_chains_state,
       GB300_energy_batch, GB300_set_mode, GB300_autotune, GB300_chains_log, GB300_chains_snapshot,
       GB300_chains_restore, GB300_chains_coeff, GB300_chains_destroy, GB300_chains_set_move,
       GB300_chains_enable_move_log, GB300_mlp_create, GB300_mlp_destroy, GB300_set_angular,
       GB300_createSphericalHarmonicsStructure, GB300_fitStructures_random, GB300_retrieveSolution

const libtp3 = joinpath(@__DIR__, "..", "lib", "libtp3.so")

const TP3_OK = Int32(0)

function check(status::Int32, ctx::Ptr{Void})
    if status != TP3_OK
        msg = unsafe_string(ccall((:tp3_last_error, libtp3), Cstring, (Ptr{Void},), ctx))
        what = unsafe_string(ccall((:tp3_status_string, libtp3), Cstring, (Int32,), status))
        error("libtp3 status $status ($what): $msg")   # no CPU fallback
    end
end

"""Device-resident basis (role of BasisTypeCuda, src/cuda.jl:24-42): the fields the
annealing code reads, plus the libtp3 context that owns every device table."""
type BasisTypeGB300 <: AbstractBasisType
    ctx::Ptr{Void}
    basislen::Int64
    N::Int64
    L::Int64
    LMAX::Int64
    lrange::StepRange
    ctr::Dict
    rtc::Dict
    K::Int64
    lambda::Float64
    dq::Float64
    histogram::Any          # the c3ref last uploaded (compared by identity)
end

"""complexBasis_choice replacement (src/correlations.jl:87, src/cuda.jl:57-71)."""
function GB300_calculate_basis(L::Int64, LMAX::Int64, N::Int64, K::Int64, lambda::Float64=0.0,
                               dq::Float64=0.0, forIntensity=true)
    forIntensity || error("only the intensity basis (lrange = 0:2:L) is on the GB300 path")
    ctx = Ref{Ptr{Void}}(C_NULL)
    check(ccall((:tp3_ctx_create, libtp3), Int32,
                (Int32, Int32, Int32, Int32, Float64, Float64, Ref{Ptr{Void}}),
                L, LMAX, N, K, lambda, dq, ctx), C_NULL)
    info = zeros(Int64, 8)
    check(ccall((:tp3_basis_info, libtp3), Int32,
                (Int32, Int32, Int32, Int32, Float64, Float64, Ptr{Int64}),
                L, LMAX, N, K, lambda, dq, info), C_NULL)
    lrange = 0:2:L
    ctr = Dict(l => Umat(l) for l = lrange)
    rtc = Dict(l => ctranspose(ctr[l]) for l = lrange)
    b = BasisTypeGB300(ctx[], info[1], N, L, LMAX, lrange, ctr, rtc, K, lambda, dq, nothing)
    finalizer(b, x -> ccall((:tp3_ctx_destroy, libtp3), Void, (Ptr{Void},), x.ctx))
    return b
end

"""First K shells as one contiguous K x LMAX^2 block (the layout cuda.jl:79 builds)."""
function pack(intensity::SphericalHarmonicsVolume, basis::BasisTypeGB300)
    n = num_coeff(basis.LMAX)
    buf = Array{Complex{Float64}}(n, basis.K)
    for k = 1:basis.K
        buf[:, k] = intensity.coeff[k][1:n]
    end
    return buf
end

"""src/cuda.jl:74-108 on libtp3 (tp3_c3)."""
function FullCorrelation_parallized(intensity::SphericalHarmonicsVolume, basis::BasisTypeGB300,
                                    minimal::Bool=true, normalize::Bool=false, return_raw::Bool=false)
    klength = div(basis.K * (basis.K + 1) * (basis.K + 2), 6)
    raw = Array{Float32}(2 * basis.N^2, klength)
    check(ccall((:tp3_c3, libtp3), Int32, (Ptr{Void}, Ptr{Complex{Float64}}, Ptr{Float32}),
                basis.ctx, pack(intensity, basis), raw), basis.ctx)
    res = convert(Array{Float64}, raw)
    if return_raw return res end
    t = zeros(Float64, basis.N, 2 * basis.N, basis.K, basis.K, basis.K)
    i = 1
    for k1 = 1:basis.K for k2 = 1:k1 for k3 = 1:k2
        t[:, :, k3, k2, k1] = reshape(res[:, i], basis.N, 2 * basis.N)
        i += 1
    end end end
    return normalize ? t / sum(abs, t) : t
end

function set_histogram!(basis::BasisTypeGB300, c3ref::C3)
    if basis.histogram !== c3ref
        K3 = size(c3ref, 3)
        check(ccall((:tp3_set_histogram, libtp3), Int32, (Ptr{Void}, Ptr{Float64}, Int32),
                    basis.ctx, c3ref, K3), basis.ctx)
        basis.histogram = c3ref
    end
end

"""src/correlations.jl:201-226 on libtp3 (tp3_energy)."""
function energy(intensity::SphericalHarmonicsVolume, basis::BasisTypeGB300, c3ref::C3,
                K3_range::UnitRange{Int64}, measure::String="Bayes", negativity_factor::Float64=0.0)
    K3_range == 1:basis.K || error("K3_range must be 1:K")
    measure == "Bayes" || return 0.0
    set_histogram!(basis, c3ref)
    E = Ref{Float64}(0.0)
    check(ccall((:tp3_energy, libtp3), Int32, (Ptr{Void}, Ptr{Complex{Float64}}, Ref{Float64}),
                basis.ctx, pack(intensity, basis), E), basis.ctx)
    return E[]
end

energy(intensity::SphericalHarmonicsVolume, basis::BasisTypeGB300, c3ref::C3, measure::String="Bayes",
       negativity_factor::Float64=0.0) = energy(intensity, basis, c3ref, 1:basis.K, measure, negativity_factor)

"""Energies of many structures in one launch sequence (the 50 energies of
calculate_temperature, src/determination.jl:244-261; tp3_energy_batch)."""
function GB300_energy_batch(intensities::Vector{SphericalHarmonicsVolume}, basis::BasisTypeGB300, c3ref::C3)
    set_histogram!(basis, c3ref)
    coeff = cat(3, [pack(s, basis) for s in intensities]...)   # LMAX^2 x K x n, column-major
    E = zeros(Float64, length(intensities))
    check(ccall((:tp3_energy_batch, libtp3), Int32, (Ptr{Void}, Int32, Ptr{Complex{Float64}}, Ptr{Float64}),
                basis.ctx, length(intensities), coeff, E), basis.ctx)
    return E
end

"""Evaluation mode: 0 plain FP32, 1 tensor-core BF16 hi/lo x3, 2 TF32 hi/lo x3, -1 the
fastest one recorded by the autotuner for this shape (tp3_set_mode)."""
GB300_set_mode(basis::BasisTypeGB300, mode::Int) =
    check(ccall((:tp3_set_mode, libtp3), Int32, (Ptr{Void}, Int32), basis.ctx, mode), basis.ctx)

"""Time every evaluation variant on n synthetic proposals and keep the fastest
(tp3_autotune); columns (mode, coupling form, angular schedule, ms per proposal)."""
function GB300_autotune(basis::BasisTypeGB300, n::Int=64)
    cap = 32
    rep = zeros(Float64, 4, cap)
    nrep = Ref{Int32}(cap)
    check(ccall((:tp3_autotune, libtp3), Int32, (Ptr{Void}, Int32, Ptr{Float64}, Ref{Int32}),
                basis.ctx, n, rep, nrep), basis.ctx)
    return rep[:, 1:min(nrep[], cap)]
end

"""Angular-stage schedule of the tensor-core path (tp3_set_angular): 1 persistent
(default), 0 one CTA per tile."""
GB300_set_angular(basis::BasisTypeGB300, schedule::Int) =
    check(ccall((:tp3_set_angular, libtp3), Int32, (Ptr{Void}, Int32), basis.ctx, schedule), basis.ctx)

"""createSphericalHarmonicsStructure (src/structure.jl:125-134) on the GPU through
tp3_structure_sh (route 1: density -> transform -> spherical Bessel transform ->
absoluteSquare); returns (density, fourierTransform, intensity) like the reference."""
function GB300_createSphericalHarmonicsStructure(basis::BasisTypeGB300, moleculepdb, LMAX::Integer,
                                                 KMAX::Integer, rmax::Float64)
    atomlist = loadPDB(moleculepdb)
    atoms = zeros(Float64, 5, length(atomlist))
    for (i, a) in enumerate(atomlist)
        f = atomfactorlist[a.t]
        atoms[:, i] = [a.pos[1], a.pos[2], a.pos[3], f.R, f.B]
    end
    start = Int32[0, length(atomlist)]
    out = [zeros(Complex{Float64}, LMAX^2, KMAX) for _ = 1:3]
    check(ccall((:tp3_structure_sh, libtp3), Int32,
                (Ptr{Void}, Ptr{Float64}, Ptr{Int32}, Int32, Int32, Int32, Float64, Int32,
                 Ptr{Complex{Float64}}, Ptr{Complex{Float64}}, Ptr{Complex{Float64}}),
                basis.ctx, atoms, start, 1, LMAX, KMAX, rmax, 1, out[1], out[2], out[3]), basis.ctx)
    qmax = pi * KMAX / rmax
    vol(c, r) = SphericalHarmonicsVolume([c[:, k] for k = 1:KMAX], LMAX, KMAX, r)
    return vol(out[1], rmax), vol(out[2], qmax), vol(out[3], qmax)
end

"""fitStructures_random (src/data_processing.jl:51-75) on the GPU (tp3_fit_structures_random)
for a volume of the basis's shape; returns (rotated volume, similarity, theta, phi, gamma)."""
function GB300_fitStructures_random(basis::BasisTypeGB300, volume::SphericalHarmonicsVolume,
                                    reference::SphericalHarmonicsVolume, K_range::UnitRange{Int64}, L::Int64,
                                    stepsizefactor::Float64, repititions::Int64=4)
    S = 0
    st = pi
    while st > pi / 180.0
        S += 1
        st *= stepsizefactor
    end
    draws = zeros(Float64, 3 + 3 * S, repititions)
    for r = 1:repititions
        draws[1:3, r] = rand(3)
        draws[4:end, r] = randn(3 * S)
    end
    vol = hcat(volume.coeff[1:basis.K]...)
    ref = hcat(reference.coeff[1:basis.K]...)
    best = zeros(Float64, 4)
    rotated = similar(vol)
    check(ccall((:tp3_fit_structures_random, libtp3), Int32,
                (Ptr{Void}, Ptr{Complex{Float64}}, Ptr{Complex{Float64}}, Int32, Int32, Int32, Float64, Int32,
                 Ptr{Float64}, Ptr{Float64}, Ptr{Complex{Float64}}),
                basis.ctx, vol, ref, first(K_range), last(K_range), L, stepsizefactor, repititions, draws, best,
                rotated), basis.ctx)
    out = SphericalHarmonicsVolume([rotated[:, k] for k = 1:basis.K], volume.LMAX, basis.K, volume.rmax)
    return out, best[1], best[2], best[3], best[4]
end

"""retrieveSolution (src/correlations.jl:261-319) on the GPU (tp3_retrieve_solution): c2 is
the reference's C2 array (N x K2 x K2, alpha first); returns the intensity volume."""
function GB300_retrieveSolution(basis::BasisTypeGB300, c2::Array{Float64,3}, L::Int64, LMAX::Int64,
                                K2_range::UnitRange{Int64}, qmax::Float64, lambda::Float64=0.0)
    N, Kd = size(c2, 1), size(c2, 2)
    c = permutedims(c2, [3, 2, 1])   # row-major [alpha][k2][k1] for the C side
    out = zeros(Complex{Float64}, LMAX^2, last(K2_range))
    check(ccall((:tp3_retrieve_solution, libtp3), Int32,
                (Ptr{Void}, Ptr{Float64}, Int32, Int32, Int32, Int32, Int32, Int32, Float64, Float64,
                 Ptr{Complex{Float64}}),
                basis.ctx, c, N, Kd, L, LMAX, first(K2_range), last(K2_range), qmax, lambda, out), basis.ctx)
    return SphericalHarmonicsVolume([out[:, k] for k = 1:last(K2_range)], LMAX, last(K2_range), qmax)
end

# ---- device-resident chains (rotate_all_at_once on the GPU) ---------------------------
function GB300_chains_create(basis::BasisTypeGB300, starts::Vector{SphericalHarmonicsVolume}, T0::Vector{Float64},
                             initial_stepsize::Float64, stepsizefactor::Float64, temperature_decay::Float64,
                             seed::UInt64; ncand::Int=16, log_capacity::Int=0)
    coeff = cat(3, [pack(s, basis) for s in starts]...)
    h = Ref{Ptr{Void}}(C_NULL)
    check(ccall((:tp3_chains_create, libtp3), Int32,
                (Ptr{Void}, Int32, Int32, Ptr{Complex{Float64}}, Ptr{Float64}, Float64, Float64, Float64,
                 UInt64, Int32, Ref{Ptr{Void}}),
                basis.ctx, length(starts), ncand, coeff, T0, initial_stepsize, stepsizefactor,
                temperature_decay, seed, log_capacity, h), basis.ctx)
    return h[]
end

GB300_chains_run(basis::BasisTypeGB300, h::Ptr{Void}, launches::Int) =
    check(ccall((:tp3_chains_run, libtp3), Int32, (Ptr{Void}, Int32), h, launches), basis.ctx)

GB300_chains_destroy(h::Ptr{Void}) = ccall((:tp3_chains_destroy, libtp3), Void, (Ptr{Void},), h)

"""The last steps of one chain (the det.out columns of src/determination.jl:512-514):
8 x n rows of step, sign, E_new, E, dE, T, acceptance probability, sigma_L."""
function GB300_chains_log(basis::BasisTypeGB300, h::Ptr{Void}, chain::Int, capacity::Int)
    rows = zeros(Float64, 8, capacity)
    n = Ref{Int64}(0)
    check(ccall((:tp3_chains_log, libtp3), Int32, (Ptr{Void}, Int32, Ptr{Float64}, Ref{Int64}),
                h, chain, rows, n), basis.ctx)
    return rows[:, 1:n[]]
end

"""Current coefficients of n chains (LMAX^2 x K x n)."""
function GB300_chains_coeff(basis::BasisTypeGB300, h::Ptr{Void}, n::Int)
    c = Array{Complex{Float64}}(num_coeff(basis.LMAX), basis.K, n)
    check(ccall((:tp3_chains_coeff, libtp3), Int32, (Ptr{Void}, Ptr{Complex{Float64}}), h, c), basis.ctx)
    return c
end

"""Checkpoint of the chain set (the role of saveState, src/determination.jl:264-267)."""
function GB300_chains_snapshot(basis::BasisTypeGB300, h::Ptr{Void})
    nbytes = Ref{Csize_t}(0)
    check(ccall((:tp3_chains_snapshot, libtp3), Int32, (Ptr{Void}, Ptr{Void}, Csize_t, Ref{Csize_t}),
                h, C_NULL, 0, nbytes), basis.ctx)
    buf = zeros(UInt8, nbytes[])
    check(ccall((:tp3_chains_snapshot, libtp3), Int32, (Ptr{Void}, Ptr{UInt8}, Csize_t, Ref{Csize_t}),
                h, buf, length(buf), nbytes), basis.ctx)
    return buf
end

GB300_chains_restore(basis::BasisTypeGB300, h::Ptr{Void}, buf::Vector{UInt8}) =
    check(ccall((:tp3_chains_restore, libtp3), Int32, (Ptr{Void}, Ptr{UInt8}, Csize_t), h, buf, length(buf)),
          basis.ctx)

"""Move of a chain set: 0 the reference's get_MC_step, 1 per-shell SO(3) steps, 2 the
learned mixture (network `net` with probability p_net), Metropolis-Hastings corrected."""
GB300_chains_set_move(basis::BasisTypeGB300, h::Ptr{Void}, kind::Int, sigma0::Float64, p_net::Float64=0.0,
                      net::Ptr{Void}=C_NULL) =
    check(ccall((:tp3_chains_set_move, libtp3), Int32, (Ptr{Void}, Int32, Float64, Float64, Ptr{Void}),
                h, kind, sigma0, p_net, net), basis.ctx)

GB300_chains_enable_move_log(basis::BasisTypeGB300, h::Ptr{Void}, launches::Int) =
    check(ccall((:tp3_chains_enable_move_log, libtp3), Int32, (Ptr{Void}, Int32), h, launches), basis.ctx)

"""The proposal network (n_in = (L+1)^2 + 33 features per shell); trained from Python or
any binding of tp3_mlp_train_step."""
function GB300_mlp_create(basis::BasisTypeGB300, hidden::Int, max_rows::Int, seed::UInt64)
    n_in = (basis.L + 1)^2 + 33
    h = Ref{Ptr{Void}}(C_NULL)
    check(ccall((:tp3_mlp_create, libtp3), Int32, (Ptr{Void}, Int32, Int32, Int32, UInt64, Ref{Ptr{Void}}),
                basis.ctx, n_in, hidden, max_rows, seed, h), basis.ctx)
    return h[]
end

GB300_mlp_destroy(net::Ptr{Void}) = ccall((:tp3_mlp_destroy, libtp3), Void, (Ptr{Void},), net)

function GB300_chains_state(basis::BasisTypeGB300, h::Ptr{Void}, n::Int)
    E = zeros(n); T = zeros(n); steps = zeros(Int64, n); acc = zeros(Int64, n)
    sigma = zeros(div(basis.L, 2) + 1, n)
    check(ccall((:tp3_chains_state, libtp3), Int32,
                (Ptr{Void}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Int64}, Ptr{Int64}),
                h, E, T, sigma, steps, acc), basis.ctx)
    return E, T, sigma, steps, acc
end

end # module
