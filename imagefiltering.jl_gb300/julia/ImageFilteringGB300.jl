# ImageFilteringGB300.jl -- the Julia side of the drop-in: a new algorithm tag
# `GB300 <: ImageFiltering.Algorithm.Alg` whose backend methods `ccall` the
# C ABI of libifx_gb300.so (include/ifx_gb300.h) instead of padding a copy and
# running the CPU loops.
#
# The reference's dispatch steps 1-4 (output eltype, kernel factoring, border
# resolution, output allocation; src/imfilter.jl:1-49, 204-254) run unchanged;
# `default_resource(alg)` wraps the tag in CPU1(GB300()) (src/imfilter.jl:1273)
# and the methods below, more specific than the reference's
# `imfilter!(r::AbstractResource, ..., border::BorderSpecAny)`
# (src/imfilter.jl:321-341), take over before any padding happens.
#
# Status: written against ImageFiltering.jl v0.7.12; it cannot be executed in
# the build environment of this package (no Julia toolchain there).
module ImageFilteringGB300

using ImageFiltering, ComputationalResources, OffsetArrays, Statistics
using ImageFiltering: ProcessedKernel, ReshapedOneD, Pad, Fill, NoPad, Inner, NA, BorderSpecAny, iscopy
using ImageFiltering.Algorithm: Alg
using ImageCore: N0f8, N0f16, Gray, Normed

export GB300

const libifx = get(ENV, "IFX_GB300_LIB", joinpath(@__DIR__, "..", "_build", "libifx_gb300.so"))

"Filter on a GB300 GPU (sm_103a kernels of libifx_gb300)."
struct GB300 <: Alg end

# ---------------------------------------------------------------- C structs
struct IfxArray
    data::Ptr{Cvoid}
    eltype::Int32
    ndim::Int32
    size::NTuple{4,Int64}
    stride::NTuple{4,Int64}
    first::NTuple{4,Int64}
end

struct IfxBorder
    style::Int32
    explicit_pad::Int32
    lo::NTuple{4,Int64}
    hi::NTuple{4,Int64}
    fill_value::Float64
end

struct IfxFactor
    axis::Int32
    length::Int32
    first::Int64
    weights::Ptr{Float64}
end

const IFX_OK = 0
eltcode(::Type{Float32}) = Int32(0)
eltcode(::Type{Float64}) = Int32(1)
eltcode(::Type{<:Union{N0f8,Gray{N0f8}}}) = Int32(2)
eltcode(::Type{UInt8}) = Int32(3)
eltcode(::Type{Int16}) = Int32(4)
eltcode(::Type{Gray{T}}) where {T<:Union{Float32,Float64}} = eltcode(T)
eltcode(::Type{Int8}) = Int32(5)
eltcode(::Type{UInt16}) = Int32(6)
eltcode(::Type{Int32}) = Int32(7)
eltcode(::Type{Int64}) = Int32(8)
eltcode(::Type{<:Union{N0f16,Gray{N0f16}}}) = Int32(9)

# Eltypes the filters read directly; the others (Int8 .. Int64, UInt16,
# Gray{N0f16}) go through ifx_convert (filter_converted! below).
native(::Type{T}) where {T} = T <: Union{Float32,Float64,N0f8,Gray{N0f8},UInt8,Gray{Float32},Gray{Float64}}

npre(::ReshapedOneD{T,N,Npre}) where {T,N,Npre} = Npre     # the axis a factor filters (0-based)

pad4(t, v) = ntuple(d -> d <= length(t) ? Int64(t[d]) : Int64(v), 4)

function ifxarray(A::AbstractArray{T,N}) where {T,N}
    N <= 4 || throw(ArgumentError("at most 4 dimensions"))
    P = parent(A)
    IfxArray(Ptr{Cvoid}(pointer(P)), eltcode(T), Int32(N), pad4(size(A), 1), pad4(strides(P), 0),
             pad4(map(first, axes(A)), 1))
end

const STYLES = Dict(:replicate => 0, :circular => 1, :symmetric => 2, :reflect => 3)

function ifxborder(b::Pad{N}) where {N}
    IfxBorder(Int32(STYLES[b.style]), Int32(N > 0), pad4(b.lo, 0), pad4(b.hi, 0), 0.0)
end
function ifxborder(b::Fill{T,N}, ::Type{E}) where {T,N,E}
    v = convert(E, b.value)             # BorderArray's conversion (src/borderarray.jl:11-20)
    IfxBorder(Int32(4), Int32(N > 0), pad4(b.lo, 0), pad4(b.hi, 0), Float64(real(v)))
end
ifxborder(b::Pad, ::Type) = ifxborder(b)

# ---------------------------------------------------------------- context
const CTX = Ref{Ptr{Cvoid}}(C_NULL)
function context()
    if CTX[] == C_NULL
        h = Ref{Ptr{Cvoid}}(C_NULL)
        check(ccall((:ifx_create, libifx), Cint, (Ref{Ptr{Cvoid}}, Cint), h, 0))
        CTX[] = h[]
    end
    CTX[]
end

function check(rc)
    rc == IFX_OK && return nothing
    msg = unsafe_string(ccall((:ifx_last_error, libifx), Cstring, ()))
    rc == 1 && throw(ArgumentError(msg))
    rc == 2 && throw(DimensionMismatch(msg))
    error(msg)
end

# ---------------------------------------------------------------- eltypes
"`out .= convert.(eltype(out), img)` on the GPU (ifx_convert), with Julia's InexactError."
function ifxconvert!(out::AbstractArray, img::AbstractArray)
    GC.@preserve out img begin
        rc = ccall((:ifx_convert, libifx), Cint, (Ptr{Cvoid}, Ref{IfxArray}, Ref{IfxArray}, Ptr{Cvoid}),
                   context(), Ref(ifxarray(out)), Ref(ifxarray(img)), C_NULL)
        if rc == 1 && occursin("InexactError", unsafe_string(ccall((:ifx_last_error, libifx), Cstring, ())))
            throw(InexactError(:convert, eltype(out), img))
        end
        check(rc)
    end
    out
end

# An image of an eltype the filters do not read: converted on the GPU to the
# compute type (the output's float type, Float64 for integer outputs) and
# filtered; integer results (accumfilter's promotion, src/utils.jl:124-129)
# convert back, raising InexactError as Julia's convert does.  A Fill value
# is first converted to the image's eltype (src/borderarray.jl:11-20).
function filter_converted!(r, out::AbstractArray{S,N}, img::AbstractArray{T,N}, kernel, border) where {S,T,N}
    Tc = S <: AbstractFloat ? S : Float64
    imgc = ifxconvert!(similar(img, Tc), img)
    b = border isa Fill ? Fill(Tc(convert(T, border.value)), border.lo, border.hi) : border
    S <: AbstractFloat && return imfilter!(r, out, imgc, kernel, b)
    ifxconvert!(out, imfilter!(r, similar(out, Float64), imgc, kernel, b))
end

# ---------------------------------------------------------------- imfilter!
# Separable kernels: a tuple of ReshapedOneD (KernelFactors.*) -> ifx_imfilter_factored
function ImageFiltering.imfilter!(r::CPU1{GB300}, out::AbstractArray{S,N}, img::AbstractArray{T,N},
                                  kernel::Tuple{ReshapedOneD,Vararg{ReshapedOneD}},
                                  border::Union{Pad,Fill}) where {S,T,N}
    native(T) || return filter_converted!(r, out, img, kernel, border)
    ws = [collect(Float64, parent(k.data)) for k in kernel]
    facs = [IfxFactor(Int32(npre(k)), Int32(length(k.data)),
                      Int64(first(axes(k.data, 1))), pointer(w)) for (k, w) in zip(kernel, ws)]
    b = ifxborder(border, T)
    GC.@preserve out img ws facs begin
        o, i = Ref(ifxarray(out)), Ref(ifxarray(img))
        check(ccall((:ifx_imfilter_factored, libifx), Cint,
                    (Ptr{Cvoid}, Ref{IfxArray}, Ref{IfxArray}, Int32, Ptr{IfxFactor}, Ref{IfxBorder}, Ptr{Cvoid}),
                    context(), o, i, Int32(length(facs)), facs, b, C_NULL))
    end
    out
end

# Dense kernels: the (dummy, K) pair of factorkernel or a 1-tuple -> ifx_imfilter_dense
function ImageFiltering.imfilter!(r::CPU1{GB300}, out::AbstractArray{S,N}, img::AbstractArray{T,N},
                                  kernel::Tuple{AbstractArray,Vararg{AbstractArray}},
                                  border::Union{Pad,Fill}) where {S,T,N}
    native(T) || return filter_converted!(r, out, img, kernel, border)
    ks = filter(k -> !iscopy(k), collect(kernel))
    length(ks) == 1 || throw(ArgumentError("GB300: one dense kernel per call"))
    K = ImageFiltering.samedims(out, ks[1])
    Kd = collect(Float64, parent(K))
    ksz = pad4(size(K), 1)
    kf = pad4(map(first, axes(K)), 0)
    GC.@preserve out img Kd begin
        check(ccall((:ifx_imfilter_dense, libifx), Cint,
                    (Ptr{Cvoid}, Ref{IfxArray}, Ref{IfxArray}, Ptr{Float64}, Ref{NTuple{4,Int64}},
                     Ref{NTuple{4,Int64}}, Ref{IfxBorder}, Int32, Ptr{Cvoid}),
                    context(), Ref(ifxarray(out)), Ref(ifxarray(img)), Kd, ksz, kf,
                    ifxborder(border, T), Int32(0), C_NULL))
    end
    out
end

# Laplacian stencil -> ifx_imfilter_laplacian
function ImageFiltering.imfilter!(r::CPU1{GB300}, out::AbstractArray{S,N}, img::AbstractArray{T,N},
                                  kernel::Tuple{ImageFiltering.Kernel.Laplacian},
                                  border::Union{Pad,Fill}) where {S,T,N}
    native(T) || return filter_converted!(r, out, img, kernel, border)
    flags = pad4(map(Int32, kernel[1].flags), 0)
    GC.@preserve out img begin
        check(ccall((:ifx_imfilter_laplacian, libifx), Cint,
                    (Ptr{Cvoid}, Ref{IfxArray}, Ref{IfxArray}, Ref{NTuple{4,Int32}}, Ref{IfxBorder}, Ptr{Cvoid}),
                    context(), Ref(ifxarray(out)), Ref(ifxarray(img)), map(Int32, flags),
                    ifxborder(border, T), C_NULL))
    end
    out
end

# NA() borders (src/imfilter.jl:280-318, 1094-1130): the reference's branch
# structure, with the mask, the filters and the divisions on the GPU.
const NA_CODES = Dict(isnan => Int32(0))
na_code(::NA{na}) where {na} = get(NA_CODES, na) do
    throw(ArgumentError("GB300: NA predicates are isnan, !isfinite or x->false"))
end

function ImageFiltering.imfilter!(r::CPU1{GB300}, out::AbstractArray{S,N}, img::AbstractArray{T,N},
                                  kernel::ProcessedKernel, border::NA) where {S,T,N}
    zeroed, valid = similar(out, S, axes(img)), similar(out, S, axes(img))
    has = Ref{Int32}(0)
    GC.@preserve zeroed valid img begin
        check(ccall((:ifx_na_prepare, libifx), Cint,
                    (Ptr{Cvoid}, Ref{IfxArray}, Ref{IfxArray}, Ref{IfxArray}, Int32, Ref{Int32}, Ptr{Cvoid}),
                    context(), Ref(ifxarray(zeroed)), Ref(ifxarray(valid)), Ref(ifxarray(img)),
                    T <: AbstractFloat ? na_code(border) : Int32(2), has, C_NULL))
    end
    fc = Fill(zero(S))
    if ImageFiltering.isseparable(kernel) && length(kernel) == N && has[] == 0
        imfilter!(r, out, img, kernel, fc)
        sums = [imfilter(r, fill(1.0, axes(img, d)), ImageFiltering._vec(kernel[d]), Fill(0.0)) for d in 1:N]
        descs = [ifxarray(s) for s in sums]
        GC.@preserve out sums descs begin
            check(ccall((:ifx_na_normalize_separable, libifx), Cint,
                        (Ptr{Cvoid}, Ref{IfxArray}, Ptr{IfxArray}, Ptr{Cvoid}),
                        context(), Ref(ifxarray(out)), descs, C_NULL))
        end
    else
        imfilter!(r, out, zeroed, kernel, fc)
        vp = imfilter(r, valid, kernel, Fill(zero(S)))
        GC.@preserve out vp begin
            check(ccall((:ifx_na_divide, libifx), Cint, (Ptr{Cvoid}, Ref{IfxArray}, Ref{IfxArray}, Ptr{Cvoid}),
                        context(), Ref(ifxarray(out)), Ref(ifxarray(vp)), C_NULL))
        end
    end
    out
end

# Inner(): `out` holds the interior (allocate_output, src/border.jl:687-694);
# its windows read inside `img`, so any padding gives the same values there.
function ImageFiltering.imfilter!(r::CPU1{GB300}, out::AbstractArray{S,N}, img::AbstractArray{T,N},
                                  kernel::ProcessedKernel, border::Inner) where {S,T,N}
    full = similar(img, S)
    imfilter!(r, full, img, kernel, Pad(:replicate))
    copyto!(out, CartesianIndices(axes(out)), full, CartesianIndices(axes(out)))
end

# ---------------------------------------------------------------- Algorithm.IIR()
# Triggs-Sdika cascades (src/imfilter.jl:892-1092) -> ifx_imfilter_iir.  The
# ReshapedOneD{...,TriggsSdika} tuples of IIRGaussian((σ...)) filter along their
# own axes with any Pad style (their padding is empty) or Fill; a tuple of bare
# TriggsSdika filters takes the axes in order and only :replicate or Fill.
struct IfxIir
    axis::Int32
    coef_f32::Int32
    a::NTuple{3,Float64}
    b::NTuple{3,Float64}
    scale::Float64
    M::NTuple{9,Float64}                 # row-major
    asum::Float64
    bsum::Float64
end
const TS = ImageFiltering.KernelFactors.TriggsSdika
ifxiir(k::TS{T}, axis) where {T} =
    IfxIir(Int32(axis), Int32(T === Float32), Float64.(Tuple(k.a)), Float64.(Tuple(k.b)), Float64(k.scale),
           ntuple(i -> Float64(k.M[(i - 1) ÷ 3 + 1, (i - 1) % 3 + 1]), 9), Float64(k.asum), Float64(k.bsum))

function iir_call(out, img, facs::Vector{IfxIir}, b::IfxBorder)
    GC.@preserve out img facs begin
        check(ccall((:ifx_imfilter_iir, libifx), Cint,
                    (Ptr{Cvoid}, Ref{IfxArray}, Ref{IfxArray}, Int32, Ptr{IfxIir}, Ref{IfxBorder}, Ptr{Cvoid}),
                    context(), Ref(ifxarray(out)), Ref(ifxarray(img)), Int32(length(facs)), facs, b, C_NULL))
    end
    out
end

function ImageFiltering.imfilter!(r::CPU1{GB300}, out::AbstractArray{S,N}, img::AbstractArray{T,N},
                                  kernel::Tuple{ImageFiltering.ReshapedIIR,Vararg{ImageFiltering.ReshapedIIR}},
                                  border::Union{Pad,Fill}) where {S,T,N}
    facs = [ifxiir(k.data, npre(k)) for k in kernel if !iscopy(k)]
    iir_call(out, img, facs, ifxborder(border, S))
end

function ImageFiltering.imfilter!(r::CPU1{GB300}, out::AbstractArray{S,N}, img::AbstractArray{T,N},
                                  kernel::Tuple{TS,Vararg{TS}}, border::Union{Pad,Fill}) where {S,T,N}
    isa(border, Pad) && border.style != :replicate && throw(ArgumentError("only \"replicate\" is supported"))
    length(kernel) <= N || throw(DimensionMismatch("cannot have more kernels than dimensions"))
    facs = [ifxiir(k, d - 1) for (d, k) in enumerate(kernel) if !iscopy(k)]
    iir_call(out, img, facs, ifxborder(border, S))
end

# ---------------------------------------------------------------- Algorithm.FFT()
# A second tag for the cuFFT path (src/imfilter.jl:776-884): the image padded
# to the padfft sizes and correlated with the kernelconv composite.
"Filter on a GB300 GPU through real FFTs (cuFFT)."
struct GB300FFT <: Alg end
export GB300FFT

function ImageFiltering.imfilter!(r::CPU1{GB300FFT}, out::AbstractArray{S,N}, img::AbstractArray{T,N},
                                  kernel::ProcessedKernel, border::Union{Pad{0},Fill{<:Any,0}}) where {S,T,N}
    K = ImageFiltering.samedims(out, ImageFiltering.kernelconv(kernel...))
    Kd = collect(Float64, parent(K))
    GC.@preserve out img Kd begin
        check(ccall((:ifx_imfilter_fft, libifx), Cint,
                    (Ptr{Cvoid}, Ref{IfxArray}, Ref{IfxArray}, Ptr{Float64}, Ref{NTuple{4,Int64}},
                     Ref{NTuple{4,Int64}}, Ref{IfxBorder}, Ptr{Cvoid}),
                    context(), Ref(ifxarray(out)), Ref(ifxarray(img)), Kd, pad4(size(K), 1),
                    pad4(map(first, axes(K)), 0), ifxborder(border, T), C_NULL))
    end
    out
end

# ---------------------------------------------------------------- mapwindow
# mapwindow has no Alg hook; the entry points take the resource first.
function ImageFiltering.mapwindow(r::CPU1{GB300}, f::Union{typeof(median!),typeof(median)}, img::AbstractArray{T,N},
                                  window::Dims{N}; border="replicate") where {T,N}
    # other eltypes: the median of the values converted to middle's eltype
    # (an order-preserving conversion), through ifx_convert
    if !native(T)
        M = typeof(Statistics.middle(first(img)))
        b = border isa Fill ? Fill(M(convert(T, border.value)), border.lo, border.hi) : border
        return mapwindow(r, f, ifxconvert!(similar(img, M), img), window; border=b)
    end
    wf = pad4(map(w -> -(w >> 1), window), 0)
    wl = pad4(window, 1)
    out = similar(img, typeof(Statistics.middle(first(img))))
    b = border isa AbstractString ? ImageFiltering.borderinstance(border) : border
    GC.@preserve out img begin
        check(ccall((:ifx_mapwindow_median, libifx), Cint,
                    (Ptr{Cvoid}, Ref{IfxArray}, Ref{IfxArray}, Ref{NTuple{4,Int64}}, Ref{NTuple{4,Int64}},
                     Ref{IfxBorder}, Ptr{Cvoid}),
                    context(), Ref(ifxarray(out)), Ref(ifxarray(img)), wf, wl, ifxborder(b, T), C_NULL))
    end
    out
end

ifxborder(b, ::Type) = throw(ArgumentError("GB300: borders of type $(typeof(b)) are not taken here"))

# An array of Tuple{E,E} (min, max) pairs as ifx_mapwindow_extrema writes it:
# eltype E, strides counted in pairs.
function pairout(A::AbstractArray{<:Tuple,N}, ::Type{E}) where {N,E}
    P = parent(A)
    IfxArray(Ptr{Cvoid}(pointer(P)), eltcode(E), Int32(N), pad4(size(A), 1), pad4(strides(P), 0),
             pad4(map(first, axes(A)), 1))
end
# The same pairs as the (2, size...) array of their values, element type C.
function pairvalues(A::AbstractArray{<:Tuple,N}, ::Type{C}) where {N,C}
    N <= 3 || throw(ArgumentError("GB300: at most 3 dimensions here"))
    P = parent(A)
    IfxArray(Ptr{Cvoid}(pointer(P)), eltcode(C), Int32(N + 1), pad4((2, size(A)...), 1),
             pad4((1, map(s -> 2s, strides(P))...), 0), pad4((1, map(first, axes(A))...), 1))
end

codetype(::Type{T}) where {T} = T
codetype(::Type{<:Union{N0f16,Gray{N0f16}}}) = UInt16

# mapwindow(extrema / minimum / maximum, img, window; border) ->
# ifx_mapwindow_extrema.  Without a border keyword extrema is the reference's
# Lemire filter (src/mapwindow.jl:337-338: truncated windows, even lengths
# allowed); with one, or for minimum / maximum, the generic window path
# (src/mapwindow.jl:270-333, default border "replicate").
function ImageFiltering.mapwindow(r::CPU1{GB300}, f::Union{typeof(extrema),typeof(minimum),typeof(maximum)},
                                  img::AbstractArray{T,N}, window::Dims{N}; border=nothing) where {T,N}
    which = f === extrema ? Int32(0) : f === minimum ? Int32(1) : Int32(2)
    native(T) || return extrema_converted(r, f, img, window, border, which)
    lemire = which == 0 && border === nothing
    lemire || all(isodd, window) || error("entries in window must be odd, got $window")
    b = border === nothing ? ImageFiltering.borderinstance("replicate") :
        border isa AbstractString ? ImageFiltering.borderinstance(border) : border
    bref = Ref(ifxborder(b, T))
    out = similar(img, which == 0 ? Tuple{T,T} : T)
    o = which == 0 ? pairout(out, T) : ifxarray(out)
    GC.@preserve out img bref begin
        bp = lemire ? Ptr{IfxBorder}(C_NULL) : Base.unsafe_convert(Ptr{IfxBorder}, bref)
        check(ccall((:ifx_mapwindow_extrema, libifx), Cint,
                    (Ptr{Cvoid}, Ref{IfxArray}, Ref{IfxArray}, Ref{NTuple{4,Int64}}, Ref{NTuple{4,Int64}},
                     Ptr{IfxBorder}, Int32, Ptr{Cvoid}),
                    context(), Ref(o), Ref(ifxarray(img)), pad4(map(w -> -(w >> 1), window), 0), pad4(window, 1),
                    bp, which, C_NULL))
    end
    out
end

# Extrema of eltypes the kernels do not read: the values (N0f16: the codes,
# whose order is the values') converted exactly to Float64 on the GPU,
# filtered there, and converted back to the image's eltype.
function extrema_converted(r, f, img::AbstractArray{T,N}, window, border, which) where {T,N}
    C = codetype(T)
    T === Int64 && any(x -> abs(x) >= 2^53, img) &&
        throw(ArgumentError("GB300: Int64 rank filters with values beyond 2^53"))
    tmp = ifxconvert!(similar(img, Float64), C === T ? img : reinterpret(C, img))
    res = if border === nothing
        mapwindow(r, f, tmp, window)
    else
        bi = border isa AbstractString ? ImageFiltering.borderinstance(border) : border
        b = bi isa Fill ? Fill(Float64(reinterpret(C, convert(T, bi.value))), bi.lo, bi.hi) : bi
        mapwindow(r, f, tmp, window; border=b)
    end
    out = similar(img, which == 0 ? Tuple{T,T} : T)
    if which == 0
        GC.@preserve out res begin
            check(ccall((:ifx_convert, libifx), Cint, (Ptr{Cvoid}, Ref{IfxArray}, Ref{IfxArray}, Ptr{Cvoid}),
                        context(), Ref(pairvalues(out, C)), Ref(pairvalues(res, Float64)), C_NULL))
        end
    else
        ifxconvert!(C === T ? out : reinterpret(C, out), res)
    end
    out
end

# ---------------------------------------------------------------- imgradients
# imgradients has no Alg hook; this method takes the resource first.  When the
# kernel function's derivative and smoothing factors share their length and
# first index (sobel, prewitt, ando3/4/5, scharr, bickley), every gradient
# comes from one sweep (ifx_imgradients); otherwise each gradient is one
# GB300 imfilter, as the reference computes them (src/specialty.jl:39-53).
function ImageFiltering.imgradients(r::CPU1{GB300}, img::AbstractArray{T,N}, kernelfun::Function,
                                    border="replicate") where {T,N}
    extended = map(ImageFiltering.isextended, axes(img))
    kerns = ntuple(d -> kernelfun(extended, d), N)
    ax = findall(collect(extended))
    b = border isa AbstractString ? ImageFiltering.borderinstance(border) : border
    fused = native(T) && !isempty(ax) && b isa Union{Pad,Fill}
    if fused
        d1 = ax[1]
        e = length(ax) > 1 ? ax[2] : d1
        kd, ks = kerns[d1][d1].data, kerns[d1][e].data
        deriv, smooth = collect(Float64, parent(kd)), collect(Float64, parent(ks))
        f1 = first(axes(kd, 1))
        fused = length(smooth) == length(deriv) && first(axes(ks, 1)) == f1
    end
    fused || return ntuple(d -> imfilter(r, img, kerns[d], border), N)
    outs = ntuple(d -> similar(img, ImageFiltering.filter_type(img, kerns[d])), N)
    descs = [ifxarray(o) for o in outs]
    GC.@preserve outs img deriv smooth descs begin
        check(ccall((:ifx_imgradients, libifx), Cint,
                    (Ptr{Cvoid}, Ptr{IfxArray}, Ref{IfxArray}, Ptr{Float64}, Ptr{Float64}, Int32, Int64,
                     Ref{NTuple{4,Int32}}, Ref{IfxBorder}, Ptr{Cvoid}),
                    context(), descs, Ref(ifxarray(img)), deriv, smooth, Int32(length(deriv)), Int64(f1),
                    map(Int32, pad4(map(Int, extended), 0)), ifxborder(b, T), C_NULL))
    end
    outs
end

end # module
