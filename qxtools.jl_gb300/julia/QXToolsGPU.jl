"""
    QXToolsGPU

Julia binding of libqxgpu (include/qxgpu.h) through `ccall`: runs the `.qx` programmes that
QXTools' `generate_simulation_files` writes (src/simulation.jl:52-77) on a GB300, and provides
`single_amplitude(tnc, plan, amplitude)` and `run_simulation(circ; num_amplitudes, seed)` with
the reference's signatures (src/simulation.jl:86-91 and :103-136).  Those two compile the
network and plan with QXTools' own `build_compute_graph` and `generate_dsl_files` into a GPU
programme (cached per network object, plan and precision) and run the bitstrings on it.

Not exercised here (no Julia toolchain in the build or GPU images); the C ABI it binds is
tested through Python ctypes.  Leaf data comes from the `.jld2` that `generate_dsl_files` writes
(read with JLD2), from the `.npz` written by the Python mirror, or as a
Dict{String,Array{ComplexF64}}.
"""
module QXToolsGPU

import ChainRulesCore
using ChainRulesCore: NoTangent, ZeroTangent, AbstractZero, unthunk
import QXTools
import JLD2

export QxgProgram, parse_qx, load_qx, read_bitstrings, qxrun, plan_contraction, amplitudes,
       single_amplitude, run_simulation, set_leaves!, gradient, compile_tnc

const libqxgpu = joinpath(@__DIR__, "..", "_build", "libqxgpu.so")

const PREC = Dict(:fp64 => Int32(0), :split_bf16 => Int32(1), :split_tf32 => Int32(2), :fp32 => Int32(3))

struct QxgInstr            # qxg_instr
    op::Int32; dst::Int32; a::Int32; b::Int32; pos::Int32; dim::Int32
    nc::Int32; na::Int32; nb::Int32; label_off::Int32
end

struct QxgOptions          # qxg_options
    precision::Int32; device::Int32; workspace_limit::Int64
    max_bitstring_batch::Int32; max_slice_batch::Int32; use_graphs::Int32
    tc_tuning::Int32        # 0: autotune tensor-core tile variants, 1: fixed default
    tc_plane_budget_mb::Int32   # 0: 4096 MiB of packed planes before blocking the free columns
    tc_wait_limit::Int32    # 0: 2^20 polls before a tensor-core wait gives up
    tc_stall_test::Int32    # test hook, leave 0
    cuda_core_joins::Int32  # 1: final joins on the CUDA cores instead of the tensor-core join
    reserved::NTuple{2,Int32}
end

mutable struct QxgProgram
    handle::Ptr{Cvoid}
    nqubits::Int
    output_size::Int
    num_slices::Int
    keys::Vector{String}            # data keys, numbered by first `load`
    data_dims::Vector{Vector{Int}}  # dims of each data key's leaf
    load_data::Vector{Int}          # data key (1-based) of each `load` command, in programme order
end

last_error() = unsafe_string(ccall((:qxg_last_error, libqxgpu), Cstring, ()))
check(rc) = rc == 0 || error("libqxgpu status $rc: $(last_error())")

struct QxgQxSizes          # qxg_qx_sizes
    ninstr::Int32; ndata::Int32; nlabels::Int64; ndims::Int64; key_bytes::Int64
    nqubits::Int32; reserved::NTuple{3,Int32}
end

"""
    parse_qx(text) -> (instrs, labels, keys, rank, dims, nqubits)

The library's parse of `.qx` text (`qxg_parse_qx`): one `QxgInstr` per command, the concatenated
ncon labels, and per data key (in order of first `load`) its name, rank and dims.
"""
function parse_qx(text::AbstractString)
    sig = (Cstring, Ref{QxgQxSizes}, Ptr{QxgInstr}, Ptr{Int32}, Ptr{Int32}, Ptr{Int64}, Ptr{UInt8})
    sz = Ref(QxgQxSizes(0, 0, 0, 0, 0, 0, (0, 0, 0)))
    check(ccall((:qxg_parse_qx, libqxgpu), Cint, sig, text, sz, C_NULL, C_NULL, C_NULL, C_NULL, C_NULL))
    s = sz[]
    instrs = Vector{QxgInstr}(undef, s.ninstr); labs = Vector{Int32}(undef, s.nlabels)
    rank = Vector{Int32}(undef, s.ndata); dims = Vector{Int64}(undef, s.ndims)
    kbuf = Vector{UInt8}(undef, s.key_bytes)
    check(ccall((:qxg_parse_qx, libqxgpu), Cint, sig, text, sz, instrs, labs, rank, dims, kbuf))
    keys = s.ndata == 0 ? String[] : String.(split(String(kbuf[1:end-1]), '\0'))
    instrs, labs, keys, rank, dims, Int(s.nqubits)
end

"""
    load_qx(qx_file, data::Dict{String,<:AbstractArray}; precision=:fp64, device=0)

Compile a `.qx` programme (docs/src/users_guide.md:93-165) into a GPU programme: the library
parses the text (`qxg_parse_qx`), `data` supplies each key's leaf tensor, whose length must match
the dims of its `load` line.
"""
function load_qx(qx_file::String, data::AbstractDict; precision::Symbol=:fp64, device::Int=0)
    instrs, labs, dkeys, rank, dims, nq = parse_qx(read(qx_file, String))
    arrays = [ComplexF64.(vec(data[k])) for k in dkeys]
    ddims = Vector{Int}[]
    off = 0
    for (i, x) in enumerate(arrays)
        push!(ddims, Int.(dims[off+1:off+rank[i]])); off += rank[i]
        n = prod(ddims[i]; init=1)
        length(x) == n || error("data key $(dkeys[i]) has $(length(x)) elements, its load line wants $n")
    end
    loads = [Int(I.a) + 1 for I in instrs if I.op == 1]   # QXG_OP_LOAD
    opts = Ref(QxgOptions(PREC[precision], device, 0, 0, 0, 0, 0, 0, 0, 0, 0, ntuple(_ -> Int32(0), 2)))
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:qxg_program_create, libqxgpu), Cint,
                (Ptr{QxgInstr}, Int32, Ptr{Int32}, Int64, Ptr{Int32}, Ptr{Int64}, Int32, Int32,
                 Ref{QxgOptions}, Ref{Ptr{Cvoid}}),
                instrs, length(instrs), labs, length(labs), rank, dims, length(arrays), nq, opts, h))
    for (i, x) in enumerate(arrays)           # column-major ComplexF64 = interleaved doubles
        check(ccall((:qxg_program_set_data, libqxgpu), Cint, (Ptr{Cvoid}, Int32, Ptr{ComplexF64}, Int64),
                    h[], i - 1, x, length(x)))
    end
    info = zeros(UInt8, 128)                  # qxg_program_info: num_slices, output_size first
    check(ccall((:qxg_program_info_get, libqxgpu), Cint, (Ptr{Cvoid}, Ptr{UInt8}), h[], info))
    ns, osz = reinterpret(Int64, info[1:16])
    p = QxgProgram(h[], nq, osz, ns, dkeys, ddims, loads)
    finalizer(p) do p
        ccall((:qxg_program_destroy, libqxgpu), Cvoid, (Ptr{Cvoid},), p.handle)
    end
    p
end

"""
    amplitudes(p, bitstrings; slices=0:p.num_slices-1) -> Matrix{ComplexF64} (output_size x n)

Saved tensor per bitstring summed over the slice range (the `max_slices` of qxrun, bin/qxrun.jl:36-39).
"""
function amplitudes(p::QxgProgram, bitstrings::AbstractVector{<:AbstractString};
                    slices::UnitRange{Int}=0:p.num_slices-1)
    buf = Vector{UInt8}(join(bitstrings))
    out = Matrix{ComplexF64}(undef, p.output_size, length(bitstrings))
    check(ccall((:qxg_amplitudes, libqxgpu), Cint, (Ptr{Cvoid}, Ptr{UInt8}, Int32, Int64, Int64, Ptr{ComplexF64}),
                p.handle, buf, length(bitstrings), first(slices), last(slices) + 1, out))
    out
end

struct QxgYmlOutput        # qxg_yml_output
    method::Int32; num_qubits::Int32; num_samples::Int64; nbitstrings::Int64; seed::Int64
    M::Float64; has_seed::Int32; fix_M::Int32; reserved::NTuple{4,Int32}
end

"""
    read_bitstrings(yml_file) -> Vector{String}

The `List` bitstrings of a `.yml` parameter file (docs/src/users_guide.md:22-35) through the
library's reader (`qxg_parse_yml_output`).  Other output methods draw their bitstrings on the
host (QXTools' samplers), so they are an error here.
"""
function read_bitstrings(yml_file::String)
    text = read(yml_file, String)
    sig = (Cstring, Ref{QxgYmlOutput}, Ptr{UInt8}, Int64)
    o = Ref(QxgYmlOutput(0, 0, 0, 0, 0, 0.0, 0, 0, (0, 0, 0, 0)))
    check(ccall((:qxg_parse_yml_output, libqxgpu), Cint, sig, text, o, C_NULL, 0))
    o[].method == 0 || error("$yml_file: the output method is not List")
    n, q = Int(o[].nbitstrings), Int(o[].num_qubits)
    buf = Vector{UInt8}(undef, n * q)
    check(ccall((:qxg_parse_yml_output, libqxgpu), Cint, sig, text, o, buf, length(buf)))
    [String(buf[i*q+1:(i+1)*q]) for i in 0:n-1]
end

"""
    qxrun(qx_file, data, yml_file; max_slices=nothing, precision=:fp64) -> Dict{String,ComplexF64}

The `.qx` + leaf data + `.yml` run of qxrun (bin/qxrun.jl:83-87) on the GPU: one amplitude per
List bitstring, summed over the first `max_slices` slices (all when `nothing`).
"""
function qxrun(qx_file::String, data::AbstractDict, yml_file::String;
               max_slices::Union{Int,Nothing}=nothing, precision::Symbol=:fp64)
    p = load_qx(qx_file, data; precision=precision)
    bits = read_bitstrings(yml_file)
    ns = max_slices === nothing ? p.num_slices : min(max_slices, p.num_slices)
    amps = amplitudes(p, bits; slices=0:ns-1)
    Dict(b => amps[1, i] for (i, b) in enumerate(bits))
end

struct QxgPlanOptions      # qxg_plan_options
    trials::Int32; greedy_trials::Int32; seed::Int64; max_log2::Float64
    num_sliced::Int32; max_sliced::Int32; flops_per_s::Float64; bytes_per_s::Float64
    tensor_batched::Ptr{UInt8}; batch_log2::Float64; reserved::NTuple{6,Int32}
end

struct QxgPlanStats        # qxg_plan_stats
    log2_flops::Float64; log2_flops_total::Float64; max_log2::Float64; time::Float64
    log2_slices::Float64; num_sliced::Int32; trees_tried::Int32; reserved::NTuple{6,Int32}
end

"""
    plan_contraction(tensor_labels, log2dims; open=nothing, max_log2=0, num_sliced=0,
                     trials=64, seed=0, batched=nothing, batch=1) -> (steps, sliced, stats)

The library's planner (`qxg_plan_contraction`) in place of FlowCutter
(flow_cutter_contraction_plan, src/contraction_planning.jl:90-113, and the slicer of
contraction_scheme, :219-299).  `tensor_labels[i]` lists the label ids (1-based) of tensor i,
`log2dims[l]` is log2 of label l's dimension, `open[l]` keeps label l to the end.  `steps[k] =
(a, b)` contracts nodes a and b into node `length(tensor_labels) + k` (nodes 1..n are the
tensors), so naming node n+k `:I\$k` gives the reference's `(A, B, C)` plan; `sliced` lists the
labels to slice.  Steps that depend on a tensor with `batched[i]` run `batch` times in the step
model (the output tensors and the number of bitstrings).
"""
function plan_contraction(tensor_labels::AbstractVector, log2dims::AbstractVector{<:Integer};
                          open=nothing, max_log2::Real=0, num_sliced::Integer=0, trials::Integer=64,
                          seed::Integer=0, batched=nothing, batch::Integer=1)
    n, nl = length(tensor_labels), length(log2dims)
    off = Int64[0]; labs = Int32[]
    for t in tensor_labels
        append!(labs, Int32.(t) .- Int32(1)); push!(off, length(labs))
    end
    w = Int32.(log2dims)
    op = open === nothing ? zeros(UInt8, nl) : UInt8.(open)
    bt = batched === nothing ? zeros(UInt8, n) : UInt8.(batched)
    pairs = zeros(Int32, max(1, 2 * (n - 1))); sl = zeros(UInt8, max(1, nl))
    st = Ref(QxgPlanStats(0, 0, 0, 0, 0, 0, 0, ntuple(_ -> Int32(0), 6)))
    GC.@preserve bt begin
        o = Ref(QxgPlanOptions(trials, 0, seed, max_log2, num_sliced, 0, 0, 0,
                               batched === nothing ? C_NULL : pointer(bt), batch > 1 ? log2(batch) : 0,
                               ntuple(_ -> Int32(0), 6)))
        check(ccall((:qxg_plan_contraction, libqxgpu), Cint,
                    (Int32, Ptr{Int64}, Ptr{Int32}, Int32, Ptr{Int32}, Ptr{UInt8}, Ref{QxgPlanOptions},
                     Ptr{Int32}, Ptr{UInt8}, Ref{QxgPlanStats}),
                    n, off, labs, nl, w, op, o, pairs, sl, st))
    end
    steps = [(Int(pairs[2k-1]) + 1, Int(pairs[2k]) + 1) for k in 1:n-1]
    steps, findall(!iszero, sl[1:nl]), st[]
end

"""
    set_leaves!(p, leaves)

Replace the programme's leaf data (`qxg_program_set_data`): `leaves[i]` is the tensor of data key
`p.keys[i]`, with `prod(p.data_dims[i])` elements (column-major, as Julia stores it).
"""
function set_leaves!(p::QxgProgram, leaves::AbstractVector{<:AbstractArray})
    length(leaves) == length(p.keys) || error("$(length(leaves)) leaves for $(length(p.keys)) data keys")
    for (i, x) in enumerate(leaves)
        v = ComplexF64.(vec(x))
        length(v) == prod(p.data_dims[i]; init=1) ||
            error("leaf $i ($(p.keys[i])) has $(length(v)) elements, its load line wants $(prod(p.data_dims[i]; init=1))")
        check(ccall((:qxg_program_set_data, libqxgpu), Cint, (Ptr{Cvoid}, Int32, Ptr{ComplexF64}, Int64),
                    p.handle, i - 1, v, length(v)))
    end
    p
end

"""
    gradient(p, bitstrings; amp_bar=nothing, slices=0:p.num_slices-1) -> (amps, leaf_grads)

Reverse-mode pass of the programme (`qxg_gradient`): the amplitudes (output_size x n) and, per
data key, dL/d conj(leaf) with the leaf's dims, summed over every `load` of that key.
`amp_bar[:, j]` is dL/d conj(amplitude) for bitstring j; `nothing` means L = sum |amplitude|^2
(then the slice range must fit one slice batch of the programme).
"""
function gradient(p::QxgProgram, bitstrings::AbstractVector{<:AbstractString}; amp_bar=nothing,
                  slices::UnitRange{Int}=0:p.num_slices-1)
    n = length(bitstrings)
    buf = Vector{UInt8}(join(bitstrings))
    out = Matrix{ComplexF64}(undef, p.output_size, n)
    sizes = [prod(d; init=1) for d in p.data_dims]
    grads = Vector{ComplexF64}(undef, max(1, sum((sizes[d] for d in p.load_data); init=0)))
    ab = amp_bar === nothing ? nothing : Matrix{ComplexF64}(reshape(amp_bar, p.output_size, n))
    check(ccall((:qxg_gradient, libqxgpu), Cint,
                (Ptr{Cvoid}, Ptr{UInt8}, Int32, Int64, Int64, Ptr{ComplexF64}, Ptr{ComplexF64}, Ptr{ComplexF64}),
                p.handle, buf, n, first(slices), last(slices) + 1,
                ab === nothing ? Ptr{ComplexF64}(C_NULL) : ab, out, grads))
    dleaf = [zeros(ComplexF64, sizes[i]) for i in eachindex(sizes)]
    off = 0
    for d in p.load_data                      # one block per `load`, in programme order
        dleaf[d] .+= view(grads, off+1:off+sizes[d]); off += sizes[d]
    end
    out, [reshape(dleaf[i], p.data_dims[i]...) for i in eachindex(dleaf)]
end

"""
    amplitudes(p, leaves, bitstrings; slices) -> Matrix{ComplexF64}

The amplitudes with the leaf tensors as an argument (`set_leaves!`, then `amplitudes`), so that
automatic differentiation reaches them: its `ChainRulesCore.rrule` pulls the amplitudes'
cotangent back through `qxg_gradient`, and the gate angles of a parametrised circuit get their
gradients through whatever Julia code builds `leaves` from them.
"""
function amplitudes(p::QxgProgram, leaves::AbstractVector{<:AbstractArray},
                    bitstrings::AbstractVector{<:AbstractString}; slices::UnitRange{Int}=0:p.num_slices-1)
    set_leaves!(p, leaves)
    amplitudes(p, bitstrings; slices=slices)
end

# ChainRules' cotangent of a complex value z is dL/d(re z) + i dL/d(im z) = 2 dL/d conj(z).
# qxg_gradient maps dL/d conj(amplitude) to dL/d conj(leaf) linearly, so passing the amplitudes'
# cotangent as amp_bar returns the leaves' cotangent directly (both sides carry the factor 2).
function ChainRulesCore.rrule(::typeof(amplitudes), p::QxgProgram, leaves::AbstractVector{<:AbstractArray},
                              bitstrings::AbstractVector{<:AbstractString};
                              slices::UnitRange{Int}=0:p.num_slices-1)
    y = amplitudes(p, leaves, bitstrings; slices=slices)
    function amplitudes_pullback(ȳ)
        Δ = unthunk(ȳ)
        Δ isa AbstractZero && return (NoTangent(), NoTangent(), ZeroTangent(), NoTangent())
        set_leaves!(p, leaves)                # the handle may have run other leaves since
        _, g = gradient(p, bitstrings; amp_bar=Δ, slices=slices)
        dl = [eltype(leaves[i]) <: Real ? real.(reshape(g[i], size(leaves[i]))) : reshape(g[i], size(leaves[i]))
              for i in eachindex(leaves)]
        (NoTangent(), NoTangent(), dl, NoTangent())
    end
    y, amplitudes_pullback
end

# GPU programmes compiled from (network object, plan, precision, device); an entry lives as long
# as its network object
const _TNC_PROGRAMS = WeakKeyDict{Any,Dict{Any,QxgProgram}}()

"""
    compile_tnc(tnc, plan; bond_groups=nothing, precision=:fp64, device=0) -> QxgProgram

A GPU programme for a `TensorNetworkCircuit` and its `(A, B, C)` plan, built as
`generate_simulation_files` builds its files (src/simulation.jl:52-77): QXTools'
`build_compute_graph(tnc, plan, bond_groups)` (src/compute_graph/compute_graph.jl:15-98) and
`generate_dsl_files` write the `.qx` programme and the `.jld2` leaf data into a temporary
directory, which `load_qx` compiles.  The network's output tensors become the programme's
`output` commands, so one programme serves every bitstring.
"""
function compile_tnc(tnc, plan::AbstractVector; bond_groups=nothing, precision::Symbol=:fp64, device::Int=0)
    cg = QXTools.build_compute_graph(tnc, plan, bond_groups)
    mktempdir() do dir
        prefix = joinpath(dir, "programme")
        QXTools.generate_dsl_files(cg, prefix; force=true)
        data = JLD2.load(prefix * ".jld2")
        load_qx(prefix * ".qx", Dict(string(k) => v for (k, v) in data); precision=precision, device=device)
    end
end

function _tnc_programme(tnc, plan, precision::Symbol, device::Int)
    progs = get!(() -> Dict{Any,QxgProgram}(), _TNC_PROGRAMS, tnc)
    get!(progs, (hash(plan), precision, device)) do
        compile_tnc(tnc, plan; precision=precision, device=device)
    end
end

"""
    single_amplitude(tnc::TensorNetworkCircuit, plan::Vector{NTuple{3,Symbol}},
                     amplitude::Union{String,Nothing}=nothing; precision=:fp64, device=0) -> ComplexF64

The reference's `single_amplitude` (src/simulation.jl:86-91) on the GPU: the amplitude of the
bitstring `amplitude` (character i = qubit i, `0 1 + -`; `nothing` = all zeros) for the network
contracted along `plan`.  The first call for a network object and plan compiles a programme
(`compile_tnc`); later calls with other bitstrings reuse it.  The network is not modified.  A
network changed in place after its first call needs `empty!(QXToolsGPU._TNC_PROGRAMS)`.
"""
function single_amplitude(tnc::QXTools.TensorNetworkCircuit, plan::Array{NTuple{3,Symbol},1},
                          amplitude::Union{String,Nothing}=nothing; precision::Symbol=:fp64, device::Int=0)
    p = _tnc_programme(tnc, plan, precision, device)
    bits = amplitude === nothing ? "0"^p.nqubits : amplitude
    amplitudes(p, [bits])[1, 1]
end

"""
    run_simulation(circ; num_amplitudes=nothing, seed=nothing, precision=:fp64, device=0)
        -> OrderedDict{String,ComplexF64}

The reference's `run_simulation` (src/simulation.jl:103-136) on the GPU: the circuit is converted
and planned by QXTools itself (`convert_to_tnc`, `flow_cutter_contraction_plan(tnc;
hypergraph=true)`), the bitstrings are `amplitudes_all` or `amplitudes_uniform(qubits, seed,
num_amplitudes)` as there (at most 1000 drawn above 30 qubits when none is given), and the unique
bitstrings run in one batched call instead of one `single_amplitude` each.
"""
function run_simulation(circ; num_amplitudes::Union{Int64,Nothing}=nothing, seed::Union{Int64,Nothing}=nothing,
                        precision::Symbol=:fp64, device::Int=0)
    tnc = QXTools.convert_to_tnc(circ)
    plan = QXTools.flow_cutter_contraction_plan(tnc; hypergraph=true)
    nq = QXTools.qubits(tnc)
    if num_amplitudes === nothing && nq > 30
        num_amplitudes = 1000
    end
    bits = num_amplitudes === nothing ? QXTools.amplitudes_all(nq) : QXTools.amplitudes_uniform(nq, seed, num_amplitudes)
    uniq = unique(collect(bits))
    p = compile_tnc(tnc, plan; precision=precision, device=device)
    amps = amplitudes(p, uniq)
    results = QXTools.OrderedDict{String,ComplexF64}()
    for (i, b) in enumerate(uniq)
        results[b] = amps[1, i]
    end
    results
end

"""
    single_amplitude(p::QxgProgram, amplitude::String) -> ComplexF64
    single_amplitude(p::QxgProgram, leaves, amplitude::String) -> ComplexF64

GPU counterpart of `single_amplitude(tnc, plan, amplitude)` (src/simulation.jl:86-91) for a
programme compiled from the same network and plan (`build_compute_graph` + `generate_dsl_files`).
The second form takes the leaf tensors and is differentiable in them (through the rrule of
`amplitudes`).
"""
single_amplitude(p::QxgProgram, amplitude::String) = amplitudes(p, [amplitude])[1, 1]
single_amplitude(p::QxgProgram, leaves::AbstractVector{<:AbstractArray}, amplitude::String) =
    amplitudes(p, leaves, [amplitude])[1, 1]

end # module
