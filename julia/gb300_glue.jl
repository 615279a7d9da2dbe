# gb300_glue.jl -- HaploADMIXTURE.jl's GPU plugin methods over libhaplo_gb300.so.
#
# Include this file inside `module HaploADMIXTURE`, in place of (or next to)
# the CUDA.jl files that the Requires hook loads (src/HaploADMIXTURE.jl:13-21):
#
#     include(joinpath(GB300_DIR, "julia", "gb300_glue.jl"))
#
# with GB300_DIR the root of this repository (or set ENV["HAPLO_GB300_LIB"] to
# the library path).  It defines a handle type, GB300Admix, and methods of the
# reference's own seams on it:
#
#   _cu_admixture_base(d, g_la, I, J) -> (d_cu, g_cu)    src/driver.jl:203-205, src/cuda/structs.jl:34-44
#   loglikelihood(d_cu, g_cu, q, p)                       src/cuda/runners.jl:13-16
#   em!(d_cu, g_cu), em_p!(d_cu, g_cu)                    src/cuda/runners.jl:45-55
#   update_q_cuda!(d_cu, g_cu), update_p_cuda!(d_cu, g_cu) src/cuda/runners.jl:71-92
#
# The handle's q/p/q_next/p_next/XtX/Xtz fields are host arrays with the
# field names of CuAdmixData (src/cuda/structs.jl:1-14), so the reference's
# call sites (src/algorithms_inner.jl, src/algorithms_outer.jl) run unchanged:
# their copyto_sync! and broadcasts move data between plain arrays, and every
# runner is one ccall.  The device-resident loop (whole fit on the GPU, two
# scalars per outer iteration to the host) is reached through the positional
# methods init_em!(d, g, iter, d_cu) / admixture_qn!(d, g, n_iter, rtol, d_cu)
# and gb300_fit!.  Every ccall's argument types follow include/haplo_gb300.h;
# a status other than 0 becomes error().

const libhx = get(ENV, "HAPLO_GB300_LIB",
                  joinpath(@__DIR__, "..", "haploadmixture.jl_gb300", "haplo_gb300", "libhaplo_gb300.so"))

# include/haplo_gb300.h: hx_opts, hx_loop_opts, hx_iter_info, hx_fit_info
struct HxOpts
    precision::Int32      # 0 = FP64 (plain), 1 = mixed
    device::Int32
    Qsec::Int32
    verbose::Int32
    rho::Float64
    pseudocount::Float64
    path::Int32           # 0 = tensor-core passes (mixed), 1 = CUDA cores only
    reserved::Int32
end

struct HxLoopOpts
    fix_q::Int32
    fix_p::Int32
    guarantee_increase::Int32
    penalty::Int32        # -1 = nothing, 1 = true, 0 = false
    mode::Int32           # 0 = :ZAL, 1 = :LBQN
end

struct HxIterInfo
    iter::Int32
    accepted_qn::Int32
    ll_prev::Float64
    ll_basic::Float64
    ll_qn::Float64
    ll_new::Float64
    reldiff::Float64
    seconds::Float64
end

struct HxFitInfo
    iters::Int32
    converged::Int32
    em_iters::Int32
    pad_::Int32
    ll::Float64
    seconds::Float64
end

mutable struct GB300Admix{T}
    ptr::Ptr{Cvoid}
    I::Int
    J::Int
    K::Int
    # host mirrors with CuAdmixData's field names (src/cuda/structs.jl:1-14)
    q::Matrix{T}
    q_next::Matrix{T}
    p::Matrix{T}
    p_next::Matrix{T}
    XtX_q::Array{T,3}
    Xtz_q::Matrix{T}
    XtX_p::Array{T,3}
    Xtz_p::Matrix{T}
end

function hxcheck(h::Ptr{Cvoid}, st::Integer)
    st == 0 && return nothing
    what = unsafe_string(ccall((:hx_status_string, libhx), Cstring, (Cint,), st))
    msg = unsafe_string(ccall((:hx_last_error, libhx), Cstring, (Ptr{Cvoid},), h))
    error("haplo_gb300: $what: $msg")
end

function gb300_opts(; precision::Symbol=:fp64, device::Integer=0, Q::Integer=3, verbose::Bool=false,
                    rho=1e7, pseudocount=1e-5, tensor_cores::Bool=true)
    HxOpts(precision === :mixed ? 1 : 0, device, Q, verbose, rho, pseudocount, tensor_cores ? 0 : 1, 0)
end

# src/driver.jl:203-205 (stub) / src/cuda/structs.jl:34-44: the device state of
# one fit.  Uploads the whole SnpArray.data matrix (as cuda/structs.jl:37), of
# which the first I individuals and first 2J SNPs are fitted.
function _cu_admixture_base(d::AdmixData2{T,T2}, g_la::SnpLinAlg{T2}, I::Int, J::Int;
                            opts::HxOpts=gb300_opts(Q=d.Q)) where {T,T2}
    data = g_la.s.data
    h = Ref{Ptr{Cvoid}}(C_NULL)
    st = ccall((:hx_create, libhx), Cint,
               (Ptr{UInt8}, Int64, Int64, Int64, Int64, Int32, Ref{HxOpts}, Ref{Ptr{Cvoid}}),
               data, size(data, 1), size(data, 2), I, J, d.K, opts, h)
    hxcheck(h[], st)
    K = d.K
    hx = GB300Admix{Float64}(h[], I, J, K, zeros(K, I), zeros(K, I), zeros(K, 4J), zeros(K, 4J),
                             zeros(K, K, I), zeros(K, I), zeros(K, K, 4J), zeros(K, 4J))
    finalizer(gb300_close!, hx)
    return hx, data            # (d_cu, g_cu); the methods below do not read g_cu
end

function gb300_close!(d_cu::GB300Admix)
    if d_cu.ptr != C_NULL
        ccall((:hx_destroy, libhx), Cint, (Ptr{Cvoid},), d_cu.ptr)
        d_cu.ptr = C_NULL
    end
    nothing
end

# ---- the runners of src/cuda/runners.jl -----------------------------------------

# src/cuda/runners.jl:13-16
function loglikelihood(d_cu::GB300Admix, g_cu, q::AbstractMatrix{Float64}, p::AbstractMatrix{Float64})
    ll = Ref(0.0)
    hxcheck(d_cu.ptr, ccall((:hx_loglikelihood, libhx), Cint,
                            (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ref{Float64}), d_cu.ptr, q, p, ll))
    ll[]
end

# src/cuda/runners.jl:45-49: raw EM numerators into q_next, p_next
function em!(d_cu::GB300Admix, g_cu)
    hxcheck(d_cu.ptr, ccall((:hx_em_accum, libhx), Cint,
                            (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
                            d_cu.ptr, d_cu.q, d_cu.p, d_cu.q_next, d_cu.p_next))
    d_cu.q_next, d_cu.p_next
end

# src/cuda/runners.jl:51-55: the P numerators only (fix_q)
function em_p!(d_cu::GB300Admix, g_cu)
    hxcheck(d_cu.ptr, ccall((:hx_em_p_accum, libhx), Cint,
                            (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
                            d_cu.ptr, d_cu.q, d_cu.p, d_cu.p_next))
    d_cu.p_next
end

# src/cuda/runners.jl:71-74
function update_q_cuda!(d_cu::GB300Admix, g_cu)
    hxcheck(d_cu.ptr, ccall((:hx_update_q_accum, libhx), Cint,
                            (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
                            d_cu.ptr, d_cu.q, d_cu.p, d_cu.XtX_q, d_cu.Xtz_q))
    nothing
end

# src/cuda/runners.jl:89-92
function update_p_cuda!(d_cu::GB300Admix, g_cu)
    hxcheck(d_cu.ptr, ccall((:hx_update_p_accum, libhx), Cint,
                            (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
                            d_cu.ptr, d_cu.q, d_cu.p, d_cu.XtX_p, d_cu.Xtz_p))
    nothing
end

# ---- device-resident loop (src/algorithms_outer.jl) ------------------------------

function gb300_set_qp!(d_cu::GB300Admix, q::AbstractMatrix{Float64}, p::AbstractMatrix{Float64})
    hxcheck(d_cu.ptr, ccall((:hx_set_qp, libhx), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}), d_cu.ptr, q, p))
end

function gb300_get_qp!(q::AbstractMatrix{Float64}, p::AbstractMatrix{Float64}, d_cu::GB300Admix; which::Integer=0)
    hxcheck(d_cu.ptr, ccall((:hx_get_qp, libhx), Cint, (Ptr{Cvoid}, Int32, Ptr{Float64}, Ptr{Float64}),
                            d_cu.ptr, which, q, p))
    q, p
end

function gb300_ll(d_cu::GB300Admix)
    ll = Ref(NaN)
    hxcheck(d_cu.ptr, ccall((:hx_get_ll, libhx), Cint, (Ptr{Cvoid}, Ref{Float64}), d_cu.ptr, ll))
    ll[]
end

# admixture_qn!/init_em! keyword options (src/algorithms_outer.jl:1-3, 38-41)
function gb300_set_loop_opts!(d_cu::GB300Admix; fix_q=false, fix_p=false, guarantee_increase=false,
                              penalty=nothing, mode=:ZAL)
    o = Ref(HxLoopOpts(fix_q, fix_p, guarantee_increase, penalty === nothing ? -1 : Int32(penalty),
                       mode === :LBQN ? 1 : 0))
    hxcheck(d_cu.ptr, ccall((:hx_set_loop_opts, libhx), Cint, (Ptr{Cvoid}, Ref{HxLoopOpts}), d_cu.ptr, o))
end

# init_em! (src/algorithms_outer.jl:1-22) with the whole EM loop on the GPU
function init_em!(d::AdmixData2, g, iter::Integer, d_cu::GB300Admix)
    gb300_set_qp!(d_cu, d.q, d.p)
    hxcheck(d_cu.ptr, ccall((:hx_init_em, libhx), Cint, (Ptr{Cvoid}, Int32), d_cu.ptr, iter))
    gb300_get_qp!(d.q, d.p, d_cu)
    d.ll_new = gb300_ll(d_cu)
    d
end

# one outer iteration of admixture_qn! (src/algorithms_outer.jl:65-171)
function gb300_qn_iteration!(d_cu::GB300Admix)
    info = Ref{HxIterInfo}()
    hxcheck(d_cu.ptr, ccall((:hx_qn_iteration, libhx), Cint, (Ptr{Cvoid}, Ref{HxIterInfo}), d_cu.ptr, info))
    info[]
end

# admixture_qn! (src/algorithms_outer.jl:38-172) with the loop on the GPU
function admixture_qn!(d::AdmixData2, g, n_iter::Integer, rtol, d_cu::GB300Admix; iter_count_offset::Integer=0)
    gb300_set_qp!(d_cu, d.q, d.p)
    info = Ref{HxFitInfo}()
    hxcheck(d_cu.ptr, ccall((:hx_admixture_qn, libhx), Cint, (Ptr{Cvoid}, Int32, Float64, Int32, Ref{HxFitInfo}),
                            d_cu.ptr, n_iter, rtol, iter_count_offset, info))
    gb300_get_qp!(d.q, d.p, d_cu)
    d.ll_new = info[].ll
    info[]
end

# _admixture_base's fit sequence (src/driver.jl:181-197): init_em! then admixture_qn!
function gb300_fit!(d::AdmixData2, d_cu::GB300Admix; n_iter::Integer=1000, rtol=1e-7, em_iters::Integer=5)
    gb300_set_qp!(d_cu, d.q, d.p)
    info = Ref{HxFitInfo}()
    hxcheck(d_cu.ptr, ccall((:hx_fit, libhx), Cint, (Ptr{Cvoid}, Int32, Float64, Int32, Ref{HxFitInfo}),
                            d_cu.ptr, n_iter, rtol, em_iters, info))
    gb300_get_qp!(d.q, d.p, d_cu)
    d.ll_new = info[].ll
    info[]
end

# ---- genotype checks, sweeps, bounded waits --------------------------------------

function gb300_census(d_cu::GB300Admix)
    counts = zeros(UInt64, 16)
    hxcheck(d_cu.ptr, ccall((:hx_census, libhx), Cint, (Ptr{Cvoid}, Ptr{UInt64}), d_cu.ptr, counts))
    counts
end

function gb300_double_missing(d_cu::GB300Admix)
    dm = zeros(Int64, d_cu.I)
    hxcheck(d_cu.ptr, ccall((:hx_double_missing, libhx), Cint, (Ptr{Cvoid}, Ptr{Int64}), d_cu.ptr, dm))
    dm
end

# grid splits of the mixed method's pass kernels, measured at the current Q/P
# (set them first, e.g. with gb300_set_qp!); later handles of the shape reuse them
function gb300_autotune!(d_cu::GB300Admix)
    chunks = zeros(Int32, 3)
    hxcheck(d_cu.ptr, ccall((:hx_autotune, libhx), Cint, (Ptr{Cvoid}, Ptr{Int32}), d_cu.ptr, chunks))
    chunks
end

function gb300_set_wait_budget!(d_cu::GB300Admix, cycles::Integer)
    hxcheck(d_cu.ptr, ccall((:hx_set_wait_budget, libhx), Cint, (Ptr{Cvoid}, Int64), d_cu.ptr, cycles))
end

# A K sweep with random restarts on one decoded genotype matrix (README.md:9
# names AIC model selection; the reference runs one K per run_admixture call).
# inits(K, r) -> (q0, p0).  Returns the fitted (q, p, info) of every fit.
function gb300_k_sweep(d_cu::GB300Admix, Ks, restarts::Integer, inits; n_iter=1000, rtol=1e-7, em_iters=5,
                       opts::HxOpts=gb300_opts())
    hs = Ptr{Cvoid}[]
    dims = Tuple{Int,Int}[]
    try
        for K in Ks, r in 1:restarts
            h = Ref{Ptr{Cvoid}}(C_NULL)
            hxcheck(d_cu.ptr, ccall((:hx_create_shared, libhx), Cint,
                                    (Ptr{Cvoid}, Int32, Ref{HxOpts}, Ref{Ptr{Cvoid}}), d_cu.ptr, K, opts, h))
            push!(hs, h[]); push!(dims, (K, r))
            q0, p0 = inits(K, r)
            hxcheck(h[], ccall((:hx_set_qp, libhx), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}), h[], q0, p0))
        end
        infos = Vector{HxFitInfo}(undef, length(hs))
        status = zeros(Int32, length(hs))
        ccall((:hx_fit_many, libhx), Cint,
              (Ptr{Ptr{Cvoid}}, Int32, Int32, Float64, Int32, Int32, Ptr{HxFitInfo}, Ptr{Int32}),
              hs, length(hs), n_iter, rtol, em_iters, 0, infos, status)
        out = []
        for (a, h) in enumerate(hs)
            hxcheck(h, status[a])
            K = dims[a][1]
            q = zeros(K, d_cu.I); p = zeros(K, 4 * d_cu.J)
            hxcheck(h, ccall((:hx_get_qp, libhx), Cint, (Ptr{Cvoid}, Int32, Ptr{Float64}, Ptr{Float64}), h, 0, q, p))
            push!(out, (K=K, restart=dims[a][2], q=q, p=p, info=infos[a]))
        end
        return out
    finally
        for h in hs
            ccall((:hx_destroy, libhx), Cint, (Ptr{Cvoid},), h)
        end
    end
end

# The `sparsity` branch of run_admixture (src/driver.jl:60-73, 84-105): AIM
# selection by sparse k-means with feature ranking on blocks of 2 SNPs over
# SnpArray.data; returns (clusters, sorted aims), 1-based like the reference.
function gb300_skfr(data::AbstractMatrix{UInt8}, I::Integer, K::Integer, sparsity::Integer;
                    max_iter::Integer=50, seed::Integer=0, device::Integer=0)
    clusters = zeros(Int32, I)
    aims = zeros(Int64, 2 * sparsity)
    iters = Ref{Int32}(0)
    wcss = Ref{Float64}(0.0)
    st = ccall((:hx_skfr, libhx), Cint,
               (Ptr{UInt8}, Int64, Int64, Int64, Int32, Int64, Int32, UInt64, Int32, Ptr{Int32}, Ptr{Int64}, Ref{Int32},
                Ref{Float64}),
               data, size(data, 1), size(data, 2), I, K, sparsity, max_iter, seed, device, clusters, aims, iters, wcss)
    st == 0 || error("haplo_gb300: hx_skfr: ", unsafe_string(ccall((:hx_status_string, libhx), Cstring, (Cint,), st)))
    clusters .+ 1, aims .+ 1
end

# Log-likelihood from device buffers that the caller owns (for example CuArray
# pointers from CUDA.jl's pool): allocates no device memory.  d_bed, d_q, d_p,
# d_ll and stream are device addresses / a CUstream handle.
function gb300_loglikelihood_noalloc!(d_ll::Ptr{Float64}, d_bed::Ptr{UInt8}, bytes_per_snp::Integer, I::Integer,
                                      J::Integer, K::Integer, d_q::Ptr{Float64}, d_p::Ptr{Float64};
                                      mixed::Bool=false, stream::Ptr{Cvoid}=C_NULL)
    st = ccall((:hx_loglikelihood_noalloc, libhx), Cint,
               (Ptr{UInt8}, Int64, Int64, Int64, Int32, Ptr{Float64}, Ptr{Float64}, Int32, Ptr{Float64}, Ptr{Cvoid}),
               d_bed, bytes_per_snp, I, J, K, d_q, d_p, mixed ? 1 : 0, d_ll, stream)
    st == 0 || error("haplo_gb300: hx_loglikelihood_noalloc: ",
                     unsafe_string(ccall((:hx_status_string, libhx), Cstring, (Cint,), st)))
    nothing
end
