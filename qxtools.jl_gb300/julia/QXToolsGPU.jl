"""
    QXToolsGPU

Julia binding of libqxgpu (include/qxgpu.h) through `ccall`: runs the `.qx` programmes that
QXTools' `generate_simulation_files` writes (src/simulation.jl:52-77) on a GB300, and provides a
`single_amplitude` with the reference's signature (src/simulation.jl:86-91).

Not exercised here (no Julia toolchain in the build or GPU images); the C ABI it binds is
tested through Python ctypes.  Leaf data is read from the `.npz` written by the Python mirror
or passed in as a Dict{String,Array{ComplexF64}} (e.g. loaded from the reference's `.jld2`).
"""
module QXToolsGPU

export QxgProgram, load_qx, amplitudes, single_amplitude

const libqxgpu = joinpath(@__DIR__, "..", "_build", "libqxgpu.so")

const OP_LOAD, OP_VIEW, OP_OUTPUT, OP_NCON, OP_SAVE = Int32(1), Int32(2), Int32(3), Int32(4), Int32(5)
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
    reserved::NTuple{5,Int32}
end

mutable struct QxgProgram
    handle::Ptr{Cvoid}
    nqubits::Int
    output_size::Int
    num_slices::Int
end

last_error() = unsafe_string(ccall((:qxg_last_error, libqxgpu), Cstring, ()))
check(rc) = rc == 0 || error("libqxgpu status $rc: $(last_error())")

labels(s) = s == "0" ? Int32[] : parse.(Int32, split(s, ","))

"""
    load_qx(qx_file, data::Dict{String,<:AbstractArray}; precision=:fp64, device=0)

Compile a `.qx` programme (docs/src/users_guide.md:93-165) into a GPU programme.
"""
function load_qx(qx_file::String, data::AbstractDict; precision::Symbol=:fp64, device::Int=0)
    ids = Dict{String,Int32}(); dkeys = String[]; instrs = QxgInstr[]; labs = Int32[]; nq = 0
    tid(s) = get!(ids, s, Int32(length(ids)))
    did(s) = (i = findfirst(==(s), dkeys); i === nothing ? (push!(dkeys, s); Int32(length(dkeys) - 1)) : Int32(i - 1))
    for line in eachline(qx_file)
        (isempty(strip(line)) || startswith(line, "#")) && continue
        t = split(line)
        if t[1] == "load"
            push!(instrs, QxgInstr(OP_LOAD, tid(t[2]), did(t[3]), 0, 0, 0, 0, 0, 0, 0))
        elseif t[1] == "view"
            src = ids[t[3]]
            push!(instrs, QxgInstr(OP_VIEW, tid(t[2]), src, parse(Int32, t[4][2:end]) - 1,
                                   parse(Int32, t[5]) - 1, parse(Int32, t[6]), 0, 0, 0, 0))
        elseif t[1] == "output"
            q = parse(Int32, t[3]); nq = max(nq, q)
            push!(instrs, QxgInstr(OP_OUTPUT, tid(t[2]), q - 1, parse(Int32, t[4]), 0, 0, 0, 0, 0, 0))
        elseif t[1] == "ncon"
            lc, la, lb = labels(t[3]), labels(t[5]), labels(t[7])
            a, b = ids[t[4]], ids[t[6]]
            off = Int32(length(labs)); append!(labs, lc, la, lb)
            push!(instrs, QxgInstr(OP_NCON, tid(t[2]), a, b, 0, 0, length(lc), length(la), length(lb), off))
        elseif t[1] == "save"
            push!(instrs, QxgInstr(OP_SAVE, 0, ids[t[3]], 0, 0, 0, 0, 0, 0, 0))
        else
            error("unknown .qx instruction $(t[1])")
        end
    end
    arrays = [ComplexF64.(data[k]) for k in dkeys]
    rank = Int32[ndims(x) for x in arrays]
    dims = Int64[d for x in arrays for d in size(x)]
    opts = Ref(QxgOptions(PREC[precision], device, 0, 0, 0, 0, 0, 0, ntuple(_ -> Int32(0), 5)))
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
    p = QxgProgram(h[], nq, osz, ns)
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

"""
    single_amplitude(p::QxgProgram, amplitude::String) -> ComplexF64

GPU counterpart of `single_amplitude(tnc, plan, amplitude)` (src/simulation.jl:86-91) for a
programme compiled from the same network and plan (`build_compute_graph` + `generate_dsl_files`).
"""
single_amplitude(p::QxgProgram, amplitude::String) = amplitudes(p, [amplitude])[1, 1]

end # module
