"""
    ParallelTemperingMonteCarloGB300

Julia binding of libptmc_gb300.so: `ptmc_run!` with the signature of
ParallelTemperingMonteCarlo.jl (`src/MCRun.jl:363-375`), taking the reference's
own `MCParams`, `TempGrid`, `NVT`/`NPT`, `ELJPotential(Even)`,
`EmbeddedAtomPotential` and `Config` values, running the replica cycles on the
GPU and returning an `Output` filled like `finalise_results`
(`src/Sampling.jl:377-399`).

Untested in this repository (no Julia toolchain was available); the C ABI it
calls is exercised through Python ctypes in `tests/`.
"""
module ParallelTemperingMonteCarloGB300

using ParallelTemperingMonteCarlo
using DelimitedFiles

const libptmc = joinpath(@__DIR__, "..", "_build", "libptmc_gb300.so")

# mirrors `struct ptmc_params` of include/ptmc_gb300.h (field order and C types)
struct PTMCParams
    n_runs::Cint
    n_traj::Cint
    mc_cycles::Clonglong
    eq_cycles::Clonglong
    mc_sample::Cint
    n_adjust::Cint
    n_bin::Cint
    min_acc::Cdouble
    max_acc::Cdouble
    ensemble::Cint
    pressure::Cdouble
    t_i::Cdouble
    t_f::Cdouble
    tdistr::Cint
    exch_prob::Cdouble
    precision::Cint
    resync_every::Cint
    seed::UInt64
    cycles_per_launch::Cint
    device::Cint
end

# mirrors `struct ptmc_output`
struct PTMCOutput
    en_avg::Ptr{Cdouble}
    heat_cap::Ptr{Cdouble}
    count_stat_atom::Ptr{Cdouble}
    count_stat_vol::Ptr{Cdouble}
    count_stat_exc::Ptr{Cdouble}
    max_displ::Ptr{Cdouble}
    en_histogram::Ptr{Cdouble}
    ev_histogram::Ptr{Cdouble}
    hist_params::NTuple{6,Cdouble}
    rdf::Ptr{Cdouble}
    delta_r2::Cdouble
end

# mirrors `struct ptmc_surrogate_cfg`
struct PTMCSurrogateCfg
    r_lo::Cdouble
    r_hi::Cdouble
    gamma::Cdouble
    r_cut::Cdouble
    escale::Cdouble
end

check(rc, ctx) = rc == 0 || error(unsafe_string(ccall((:ptmc_last_error, libptmc), Cstring, (Ptr{Cvoid},), ctx)))

"""
    ptmc_run!(mc_params, temp, start_config, potential, ensemble; save=false,
              precision=:fp64, exch_prob=0.1, seed=1234, resync_every=1000)

Drop-in for `ParallelTemperingMonteCarlo.ptmc_run!` on the GPU.  Returns
`(states, results)` where `states` holds slot-ordered `(config, en_tot,
max_displ)` and `results::Output`.
"""
function ptmc_run!(mc_params::MCParams, temp::TempGrid, start_config, potential, ensemble;
                   save=false, precision=:fp64, exch_prob=0.1, seed=1234, resync_every=1000,
                   rdfsave=false, workingdirectory=pwd())
    configs = start_config isa Config ? (start_config,) : Tuple(start_config)
    R = mc_params.n_traj
    N = length(configs[1])
    npt = ensemble isa NPT
    p = PTMCParams(1, R, mc_params.mc_cycles, mc_params.eq_cycles, mc_params.mc_sample,
                   mc_params.n_adjust, mc_params.n_bin, mc_params.min_acc, mc_params.max_acc,
                   npt ? 1 : (ensemble isa NNVT ? 2 : 0), npt ? ensemble.pressure : 0.0,
                   first(temp.t_grid), last(temp.t_grid), 0, exch_prob,
                   precision == :fp64 ? 0 : 1, resync_every, UInt64(seed), 0, 0)
    ctx = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:ptmc_create, libptmc), Cint, (Ptr{Ptr{Cvoid}}, Ref{PTMCParams}), ctx, p), C_NULL)
    c = ctx[]
    try
        if potential isa ELJPotentialEven || potential isa ELJPotential
            coeff = collect(Float64, potential.coeff)
            check(ccall((:ptmc_set_potential_elj, libptmc), Cint, (Ptr{Cvoid}, Ptr{Cdouble}, Cint, Cint),
                        c, coeff, length(coeff), potential isa ELJPotentialEven), c)
        elseif potential isa RuNNerPotential
            # sf rows {kind, type, eta, lambda, zeta, r_cut, G_min, G_max}: the structs keep
            # G_norm = 1/(max-min), G_offset = -min G_norm, tpz = 2^(1-zeta) G_norm
            rows = Float64[]
            for f in potential.radsymfunctions
                gmin = -f.G_offset / f.G_norm
                append!(rows, [0, f.type_vec, f.eta, 0, 0, f.r_cut, gmin, gmin + 1 / f.G_norm])
            end
            for f in potential.angsymfunctions
                gnorm = f.tpz / 2.0^(1 - f.zeta)
                gmin = -f.G_offset / gnorm
                append!(rows, [1, f.type_vec, f.eta, f.lambda, f.zeta, f.r_cut, gmin, gmin + 1 / gnorm])
            end
            nnp = potential.nnp  # parameters: per layer W[n_in][n_out] then b[n_out]
            nodes = Cint.(nnp.num_nodes)
            check(ccall((:ptmc_set_potential_nn, libptmc), Cint,
                        (Ptr{Cvoid}, Ptr{Cdouble}, Cint, Ptr{Cdouble}, Cint, Ptr{Cint}, Cint, Cdouble),
                        c, rows, length(rows) ÷ 8, nnp.parameters, length(nnp.parameters), nodes,
                        length(nodes), sqrt(potential.boundary)), c)
        elseif potential isa RuNNerPotential2Atom
            # RadialType2a / AngularType3a fields as they are
            rad = reduce(vcat, [[f.eta, f.r_cut, f.G_offset..., f.G_norm...] for f in potential.radsymfunctions])
            ang = isempty(potential.angsymfunctions) ? Float64[] :
                  reduce(vcat, [[f.eta, f.lambda, f.zeta, f.r_cut, f.tpz..., f.G_offset...]
                                for f in potential.angsymfunctions])
            nodes = Cint.(potential.nnp1.num_nodes)
            n1 = typeof(potential).parameters[3]
            check(ccall((:ptmc_set_potential_nn2, libptmc), Cint,
                        (Ptr{Cvoid}, Ptr{Cdouble}, Cint, Ptr{Cdouble}, Cint, Ptr{Cdouble}, Ptr{Cdouble},
                         Cint, Ptr{Cint}, Cint, Cint),
                        c, rad, length(potential.radsymfunctions), ang, length(potential.angsymfunctions),
                        potential.nnp1.parameters, potential.nnp2.parameters,
                        length(potential.nnp1.parameters), nodes, length(nodes), n1), c)
            ensemble isa NNVT && check(ccall((:ptmc_set_atom_swaps, libptmc), Cint, (Ptr{Cvoid}, Cint),
                                             c, ensemble.n_atom_swaps), c)
        elseif potential isa ELJPotentialB
            a, b, cc = (collect(Float64, v) for v in (potential.coeff_a, potential.coeff_b, potential.coeff_c))
            check(ccall((:ptmc_set_potential_eljb, libptmc), Cint,
                        (Ptr{Cvoid}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Cint),
                        c, a, b, cc, length(cc)), c)
        elseif potential isa LookupTablePotential
            # pot.table is Matrix{Float64}(l_angle, l_dist): passed as is (column-major)
            check(ccall((:ptmc_set_potential_lookup, libptmc), Cint,
                        (Ptr{Cvoid}, Ptr{Cdouble}, Cint, Cint, Cdouble, Cdouble, Cdouble, Cdouble, Cdouble),
                        c, potential.table, potential.l_angle, potential.l_dist, potential.start_dist,
                        potential.start_angle, potential.d_dist, potential.d_angle, potential.c6coeff), c)
        elseif potential isa EmbeddedAtomPotential
            check(ccall((:ptmc_set_potential_eam, libptmc), Cint,
                        (Ptr{Cvoid}, Cdouble, Cdouble, Cdouble, Cdouble),
                        c, potential.n, potential.m, potential.ean, potential.eCam), c)
        else
            error("potential $(typeof(potential)) is not supported by the GPU engine")
        end
        # 3 x N x n_start, column-major: exactly the layout of Vector{SVector{3}}
        xyz = reduce(hcat, [reduce(hcat, cf.positions) for cf in configs])
        bc = configs[1].boundary_condition
        kind, len, hgt = bc isa SphericalBC ? (0, sqrt(bc.radius2), sqrt(bc.radius2)) :
                         bc isa CubicBC ? (1, bc.box_length, bc.box_length) :
                         bc isa RectangularBC ? (2, bc.box_length, bc.box_height) :
                         (3, bc.box_length, bc.box_height)   # RhombicBC
        rdfsave && check(ccall((:ptmc_set_rdf, libptmc), Cint, (Ptr{Cvoid}, Cint), c, 1), c)
        if npt && ensemble.separated_volume
            check(ccall((:ptmc_set_separated_volume, libptmc), Cint, (Ptr{Cvoid}, Cint), c, 1), c)
        end
        check(ccall((:ptmc_set_run_configs_box, libptmc), Cint,
                    (Ptr{Cvoid}, Cint, Ptr{Cdouble}, Cint, Cint, Cint, Cdouble, Cdouble),
                    c, 0, xyz, N, length(configs), kind, len, hgt), c)
        check(ccall((:ptmc_init, libptmc), Cint, (Ptr{Cvoid},), c), c)
        check(ccall((:ptmc_equilibrate, libptmc), Cint, (Ptr{Cvoid},), c), c)
        done = 0
        if save !== false
            dir = joinpath(workingdirectory, "checkpoint")
            for m in save:save:mc_params.mc_cycles
                check(ccall((:ptmc_run_cycles, libptmc), Cint, (Ptr{Cvoid}, Clonglong), c, m - done), c)
                done = m
                check(ccall((:ptmc_checkpoint, libptmc), Cint, (Ptr{Cvoid}, Cstring), c, dir), c)
            end
        end
        check(ccall((:ptmc_run_cycles, libptmc), Cint, (Ptr{Cvoid}, Clonglong), c,
                    mc_params.mc_cycles - done), c)
        nb = mc_params.n_bin + 2
        en_avg, heat_cap = zeros(R), zeros(R)
        sa, sv, se = zeros(R), zeros(R), zeros(R)
        md = zeros(2R)
        eh = zeros(nb * R)
        ev = npt ? zeros(nb * nb * R) : zeros(1)
        rd = zeros(rdfsave ? 5 * mc_params.n_bin * R : 1)
        o = Ref(PTMCOutput(pointer(en_avg), pointer(heat_cap), pointer(sa), pointer(sv),
                           pointer(se), pointer(md), pointer(eh), pointer(ev), ntuple(_ -> 0.0, 6),
                           rdfsave ? pointer(rd) : C_NULL, 0.0))
        GC.@preserve en_avg heat_cap sa sv se md eh ev rd begin
            check(ccall((:ptmc_get_output, libptmc), Cint, (Ptr{Cvoid}, Cint, Ref{PTMCOutput}), c, 0, o), c)
        end
        hp = o[].hist_params
        results = Output{Float64}(mc_params.n_bin)
        results.en_min, results.en_max, results.v_min, results.v_max = hp[1], hp[2], hp[3], hp[4]
        results.delta_en_hist, results.delta_v_hist = hp[5], hp[6]
        if rdfsave
            results.delta_r2 = o[].delta_r2
            results.rdf = [rd[(k - 1) * 5 * mc_params.n_bin + 1:k * 5 * mc_params.n_bin] for k in 1:R]
        end
        results.en_avg, results.heat_cap = en_avg, heat_cap
        results.count_stat_atom, results.count_stat_exc = sa, se
        results.max_displ = md[1:2:end]
        # C fills [slot][bin] row-major; Julia wants one vector per slot
        results.en_histogram = [eh[(i - 1) * nb + 1:i * nb] for i in 1:R]
        if npt
            # [slot][e][v] row-major -> Matrix (e, v) per slot
            results.ev_histogram = [permutedims(reshape(ev[(i - 1) * nb * nb + 1:i * nb * nb], nb, nb))
                                    for i in 1:R]
        end
        xyzo = zeros(3 * N * R)
        en = zeros(R); box = zeros(R); mds = zeros(2R)
        counts = zeros(Clonglong, 6R); ham = zeros(2R)
        check(ccall((:ptmc_get_states, libptmc), Cint,
                    (Ptr{Cvoid}, Cint, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble},
                     Ptr{Clonglong}, Ptr{Cdouble}), c, 0, xyzo, en, box, mds, counts, ham), c)
        states = [(config=reshape(xyzo[(i - 1) * 3N + 1:i * 3N], 3, N), en_tot=en[i],
                   max_displ=mds[2i - 1:2i]) for i in 1:R]
        return states, results
    finally
        ccall((:ptmc_destroy, libptmc), Cvoid, (Ptr{Cvoid},), c)
    end
end

"""
    multihistogram_NVT(ensemble, temp, results, conv_threshold, readfile=false)

GPU multihistogram (`src/multihist_NVT.jl:95`); returns Cv on TempGrid{10R}.
"""
function multihistogram_NVT(ensemble, temp::TempGrid, results::Output, conv_threshold, readfile=false)
    R = length(temp.t_grid)
    nb = results.n_bin + 2
    h = reduce(vcat, results.en_histogram)          # row-major [slot][bin]
    T, cv = zeros(10R), zeros(10R)
    it = Ref{Cint}(0)
    rc = ccall((:ptmc_multihist_nvt, libptmc), Cint,
               (Cint, Cint, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Cdouble, Cdouble, Cdouble,
                Ptr{Cdouble}, Ptr{Cdouble}, Ref{Cint}),
               R, results.n_bin, h, collect(temp.t_grid), collect(temp.beta_grid),
               results.en_min, results.en_max, conv_threshold, T, cv, it)
    rc == 0 || error(unsafe_string(ccall((:ptmc_last_error, libptmc), Cstring, (Ptr{Cvoid},), C_NULL)))
    return cv
end

"""
    multihistogram(output, temp; outdir=pwd(), NPoints=1000)

Linear-solve multihistogram (`src/multihist.jl:437-455`) on the GPU
(`ptmc_multihist_linear`, gauge alpha[R] = 0); writes histograms.data, Sol.X,
S.data and analysis.NVT into `outdir` like the reference and returns
(energies, T, Z, Cv, dCv, U).
"""
function multihistogram(output::Output, temp::TempGrid; outdir=pwd(), NPoints=1000)
    R = length(temp.beta_grid)
    nb = output.n_bin
    h = reduce(vcat, output.en_histogram)            # row-major [slot][bin], n_bin + 2 bins
    E, S, alpha = zeros(nb), zeros(nb), zeros(R)
    T, Z, U, Cv, dCv, ST = (zeros(NPoints) for _ in 1:6)
    nk = Ref{Cint}(0)
    rc = ccall((:ptmc_multihist_linear, libptmc), Cint,
               (Cint, Cint, Ptr{Cdouble}, Ptr{Cdouble}, Cdouble, Cdouble, Cint, Ptr{Cdouble},
                Ptr{Cdouble}, Ref{Cint}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble},
                Ptr{Cdouble}, Ptr{Cdouble}, Ptr{Cdouble}),
               R, nb, Float64.(h), collect(temp.beta_grid), output.en_min, output.en_max, NPoints,
               E, S, nk, alpha, T, Z, U, Cv, dCv, ST)
    rc == 0 || error(unsafe_string(ccall((:ptmc_last_error, libptmc), Cstring, (Ptr{Cvoid},), C_NULL)))
    E, S = E[1:nk[]], S[1:nk[]]
    H = [Float64.(output.en_histogram[i][2:end-1]) ./ nb for i in 1:R]
    keep = findall(!iszero, sum(H))
    open(joinpath(outdir, "histograms.data"), "w") do f
        writedlm(f, permutedims(E))
        for i in 1:R
            writedlm(f, permutedims(H[i][keep]))
        end
    end
    open(joinpath(outdir, "Sol.X"), "w") do f
        writedlm(f, ["alpha"])
        writedlm(f, permutedims(alpha))
    end
    open(joinpath(outdir, "S.data"), "w") do f
        writedlm(f, ["E" "Entropy"])
        writedlm(f, [E S])
    end
    open(joinpath(outdir, "analysis.NVT"), "w") do f
        writedlm(f, ["T" "Z" "Cv" "dCv" "U(T)"])
        writedlm(f, [T Z Cv dCv U])
    end
    return E, T, Z, Cv, dCv, U
end

"""
    train_surrogate!(ctx; cycles=300, capacity=40000, steps=4000, batch=512, lr=2e-3,
                     calibrate=false)

Delayed-acceptance set-up on an initialised NN context (no counterpart in the
reference): capture `cycles` of exact moves, train the pair surrogate on the
GPU, enable screening. Screening strength 1 on every temperature (the standard
two-stage test) unless `calibrate` asks for the per-temperature choice of
`ptmc_surrogate_calibrate`.
"""
function train_surrogate!(ctx::Ptr{Cvoid}; cycles=300, capacity=40000, steps=4000, batch=512,
                          lr=2e-3, calibrate::Bool=false,
                          cfg=PTMCSurrogateCfg(2.0, 12.0, 0.5625, 12.0, 0.0))
    check(ccall((:ptmc_surrogate_set, libptmc), Cint,
                (Ptr{Cvoid}, Ref{PTMCSurrogateCfg}, Ptr{Cfloat}, Cint, Cint),
                ctx, cfg, C_NULL, capacity, 1), ctx)
    check(ccall((:ptmc_surrogate_record, libptmc), Cint, (Ptr{Cvoid}, Cint), ctx, 1), ctx)
    check(ccall((:ptmc_cycles_nosample, libptmc), Cint, (Ptr{Cvoid}, Clonglong), ctx, cycles), ctx)
    check(ccall((:ptmc_surrogate_record, libptmc), Cint, (Ptr{Cvoid}, Cint), ctx, 0), ctx)
    loss = Ref{Cdouble}(0)
    check(ccall((:ptmc_surrogate_train, libptmc), Cint, (Ptr{Cvoid}, Cint, Cint, Cdouble, Ref{Cdouble}),
                ctx, steps, batch, lr, loss), ctx)
    calibrate && check(ccall((:ptmc_surrogate_calibrate, libptmc), Cint,
                             (Ptr{Cvoid}, Cdouble, Cint, Ptr{Cdouble}), ctx, 0.0, 10, C_NULL), ctx)
    check(ccall((:ptmc_surrogate_enable, libptmc), Cint, (Ptr{Cvoid}, Cint), ctx, 1), ctx)
    return loss[]
end

end
