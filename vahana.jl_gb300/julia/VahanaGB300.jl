"""
    VahanaGB300

Julia binding of libvahana_gb300.so: Vahana.jl's public functions for the
transition step, with the simulation state resident on one GB300.  Agent
and edge types are ordinary isbits structs, as in Vahana; their fields are
stored as struct-of-arrays columns on the device.  A transition function
is a kernel registered in the library, named by a Symbol
(`transition_names()`), with its numeric parameters.

Written against include/vahana_gb300.h; no Julia toolchain was available
where this library was built, so this file has not been run.
"""
module VahanaGB300

export ModelTypes, register_agenttype!, register_edgetype!, register_param!,
       register_global!, create_model, create_simulation, finish_simulation!,
       copy_simulation, finish_init!, add_agent!, add_agents!, add_edge!, add_edges!,
       apply!, apply, apply_host!, mapreduce, agentstate, agentstate_flexible, edges, neighborids,
       neighborids_iter, neighborstates, neighborstates_iter, neighborstates_flexible,
       neighborstates_flexible_iter, edgestates, edgestates_iter, num_edges, has_edge, num_agents, all_agents,
       all_agentids, add_raster!, connect_raster_neighbors!, move_to!, cellid,
       rastervalues, calc_rasterstate, param, set_param!, get_global, set_global!, bind_param!,
       push_global!, disable_transition_checks, transition_names, Edge, AgentID,
       add_graph!, remove_edges!, add_agent_per_process!, write_snapshot, read_snapshot,
       prepare_apply, PreparedApply, release!, set_async!, synchronize

const LIB = get(ENV, "VAHANA_GB300_LIB",
                joinpath(@__DIR__, "..", "libvahana_gb300.so"))
const AgentID = UInt64

struct Edge{T}
    from::AgentID
    state::T
end

const HINTS = Dict(:Immortal => 0x01, :Independent => 0x02, :Stateless => 0x10,
                   :IgnoreFrom => 0x20, :SingleType => 0x40, :SingleEdge => 0x80,
                   :IgnoreSourceState => 0x100, :NumEdgesOnly => 0x200,
                   :HasEdgeOnly => 0x400)
const OPS = Dict(+ => 1, (*) => 2, max => 3, min => 4, (&) => 5, (|) => 6)

dtype(::Type{Bool}) = 1;   dtype(::Type{UInt8}) = 2;  dtype(::Type{Int8}) = 3
dtype(::Type{UInt16}) = 4; dtype(::Type{Int16}) = 5;  dtype(::Type{UInt32}) = 6
dtype(::Type{Int32}) = 7;  dtype(::Type{UInt64}) = 8; dtype(::Type{Int64}) = 9
dtype(::Type{Float32}) = 10; dtype(::Type{Float64}) = 11

function check(rc::Cint)
    rc == 0 && return nothing
    msg = unsafe_string(ccall((:vg_last_error, LIB), Cstring, ()))
    rc == 1 ? throw(AssertionError(msg)) : error("vahana_gb300 [$rc]: $msg")
end

edgeref(e::Integer) = Cint(0x10000 | e)

mutable struct ModelTypes
    h::Ptr{Cvoid}
    agents::Dict{DataType, Int}
    edges::Dict{DataType, Int}
    function ModelTypes()
        h = Ref{Ptr{Cvoid}}(C_NULL)
        check(ccall((:vg_model_create, LIB), Cint, (Ptr{Ptr{Cvoid}},), h))
        m = new(h[], Dict{DataType, Int}(), Dict{DataType, Int}())
        # simulations keep their own reference to the model's types, so the
        # handle may go before them
        finalizer(m -> m.h == C_NULL || ccall((:vg_model_destroy, LIB), Cvoid, (Ptr{Cvoid},), m.h), m)
    end
end

function fieldspec(T)
    names = [String(n) for n in fieldnames(T)]
    dts = Cint[dtype(ft) for ft in fieldtypes(T)]
    names, dts
end

"register_agenttype!(types, T, hints...) -- src/ModelTypes.jl:81-106"
function register_agenttype!(types::ModelTypes, ::Type{T}, hints...) where T
    names, dts = fieldspec(T)
    nr = Ref{Cint}(0)
    check(ccall((:vg_model_register_agenttype, LIB), Cint,
                (Ptr{Cvoid}, Cstring, Cint, Ptr{Cstring}, Ptr{Cint}, Cuint, Ptr{Cint}),
                types.h, String(nameof(T)), length(names), names, dts,
                reduce(|, (HINTS[h] for h in hints); init = 0x0), nr))
    types.agents[T] = nr[]
    types
end
register_agenttype!(T::DataType, hints...) = types -> register_agenttype!(types, T, hints...)

"register_edgetype!(types, T, hints...; target, size) -- src/ModelTypes.jl:158-230"
function register_edgetype!(types::ModelTypes, ::Type{T}, hints...;
                            target = nothing, size = 0) where T
    names, dts = fieldspec(T)
    e = Ref{Cint}(0)
    tnr = target === nothing ? 0 : types.agents[target]
    check(ccall((:vg_model_register_edgetype, LIB), Cint,
                (Ptr{Cvoid}, Cstring, Cint, Ptr{Cstring}, Ptr{Cint}, Cuint, Cint, Int64,
                 Ptr{Cint}),
                types.h, String(nameof(T)), length(names), names, dts,
                reduce(|, (HINTS[h] for h in hints); init = 0x0), tnr, size, e))
    types.edges[T] = e[]
    types
end
register_edgetype!(T::DataType, hints...; kw...) =
    types -> register_edgetype!(types, T, hints...; kw...)

register_param!(types::ModelTypes, name::Symbol, v) =
    (check(ccall((:vg_model_register_param, LIB), Cint, (Ptr{Cvoid}, Cstring, Cdouble),
                 types.h, String(name), v)); types)
register_global!(types::ModelTypes, name::Symbol, v) =
    (check(ccall((:vg_model_register_global, LIB), Cint, (Ptr{Cvoid}, Cstring, Cdouble),
                 types.h, String(name), v)); types)

"create_model(types, name) -- src/Simulation.jl:115-207"
function create_model(types::ModelTypes, name::String)
    check(ccall((:vg_model_finalize, LIB), Cint, (Ptr{Cvoid}, Cstring), types.h, name))
    types
end
create_model(name::String) = types -> create_model(types, name)

mutable struct Simulation
    h::Ptr{Cvoid}
    model::ModelTypes
    rasters::Dict{Symbol, Tuple}
end

"create_simulation(model; name) -- src/Simulation.jl:261-339"
function create_simulation(model::ModelTypes; name = "sim", stream = C_NULL)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:vg_sim_create, LIB), Cint,
                (Ptr{Cvoid}, Cstring, Ptr{Cvoid}, Ptr{Ptr{Cvoid}}), model.h, name, stream, h))
    sim = Simulation(h[], model, Dict{Symbol, Tuple}())
    finalizer(s -> s.h == C_NULL || ccall((:vg_sim_destroy, LIB), Cint, (Ptr{Cvoid},), s.h), sim)
    sim
end

"finish_simulation! -- src/Simulation.jl:551-573"
function finish_simulation!(sim::Simulation)
    check(ccall((:vg_sim_destroy, LIB), Cint, (Ptr{Cvoid},), sim.h))
    sim.h = C_NULL
    nothing
end

"copy_simulation(sim) -- src/Simulation.jl:500-510"
function copy_simulation(sim::Simulation)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:vg_sim_copy, LIB), Cint, (Ptr{Cvoid}, Ptr{Ptr{Cvoid}}), sim.h, h))
    c = Simulation(h[], sim.model, copy(sim.rasters))
    finalizer(s -> s.h == C_NULL || ccall((:vg_sim_destroy, LIB), Cint, (Ptr{Cvoid},), s.h), c)
end

"""
    set_async!(sim, on::Bool)

With `on`, apply! returns without waiting for the device; an error that a
kernel reports surfaces at the next `synchronize(sim)` or read back
(vg_sim_set_async).  Off by default: every apply! checks.
"""
set_async!(sim::Simulation, on::Bool) =
    check(ccall((:vg_sim_set_async, LIB), Cint, (Ptr{Cvoid}, Cint), sim.h, on ? 1 : 0))
synchronize(sim::Simulation) = check(ccall((:vg_sim_synchronize, LIB), Cint, (Ptr{Cvoid},), sim.h))

"finish_init!(sim) -- src/Simulation.jl:403-476 (one process)"
finish_init!(sim::Simulation) =
    check(ccall((:vg_finish_init, LIB), Cint, (Ptr{Cvoid},), sim.h))

disable_transition_checks(sim::Simulation, d::Bool) =
    check(ccall((:vg_disable_transition_checks, LIB), Cint, (Ptr{Cvoid}, Cint), sim.h, d))

columns(v::Vector{T}) where T = [T.types[i] === nothing ? nothing :
                                 [getfield(a, i) for a in v] for i in 1:fieldcount(T)]

"add_agents!(sim, agents) -- src/Agent.jl:174-180"
function add_agents!(sim::Simulation, agents::Vector{T}) where T
    cols = columns(agents)
    ptrs = Ptr{Cvoid}[pointer(c) for c in cols]
    ids = Vector{AgentID}(undef, length(agents))
    GC.@preserve cols check(ccall((:vg_add_agents, LIB), Cint,
        (Ptr{Cvoid}, Cint, UInt64, Ptr{Ptr{Cvoid}}, Ptr{UInt64}),
        sim.h, sim.model.agents[T], length(agents), ptrs, ids))
    ids
end
add_agents!(sim::Simulation, agents...) = add_agents!(sim, collect(agents))
"add_agent!(sim, agent) -- src/AgentMethods.jl:65-89"
add_agent!(sim::Simulation, a) = add_agents!(sim, [a])[1]

"add_edge!(sim, from, to, state) / add_edges! -- src/EdgeMethods.jl:388-523"
function add_edges!(sim::Simulation, from::Vector{AgentID}, to::Vector{AgentID},
                    states::Vector{T}) where T
    cols = columns(states)
    ptrs = Ptr{Cvoid}[pointer(c) for c in cols]
    GC.@preserve cols check(ccall((:vg_add_edges, LIB), Cint,
        (Ptr{Cvoid}, Cint, UInt64, Ptr{UInt64}, Ptr{UInt64}, Ptr{Ptr{Cvoid}}),
        sim.h, sim.model.edges[T], length(to), from, to,
        isempty(ptrs) ? C_NULL : ptrs))
end
add_edge!(sim::Simulation, from::AgentID, to::AgentID, s::T) where T =
    add_edges!(sim, [from], [to], [s])
add_edge!(sim::Simulation, to::AgentID, e::Edge{T}) where T = add_edge!(sim, e.from, to, e.state)
add_edges!(sim::Simulation, to::AgentID, es::Vector{Edge{T}}) where T =
    add_edges!(sim, [e.from for e in es], fill(to, length(es)), [e.state for e in es])

typeref(sim, T) = haskey(sim.model.agents, T) ? Cint(sim.model.agents[T]) :
                  edgeref(sim.model.edges[T])
refs(sim, v) = Cint[typeref(sim, T) for T in (v isa AbstractVector ? v : [v])]

"""
    apply!(sim, transition::Symbol, call, read, write; add_existing, with_edge, params)

apply! -- src/Simulation.jl:720-821.  `transition` names a kernel of the
library (the Julia closure of Vahana is replaced by a registered kernel).
"""
function apply!(sim::Simulation, f::Symbol, call, read, write;
                add_existing = [], with_edge = nothing, params = Float64[])
    c, r, w, a = refs(sim, call), refs(sim, read), refs(sim, write), refs(sim, add_existing)
    we = with_edge === nothing ? Cint(-1) : Cint(sim.model.edges[with_edge])
    check(ccall((:vg_apply, LIB), Cint,
                (Ptr{Cvoid}, Cstring, Ptr{Cint}, Cint, Ptr{Cint}, Cint, Ptr{Cint}, Cint,
                 Ptr{Cint}, Cint, Cint, Ptr{Cdouble}, Cint),
                sim.h, String(f), c, length(c), r, length(r), w, length(w), a, length(a), we,
                Float64.(params), length(params)))
    sim
end
apply(sim::Simulation, f::Symbol, call, read, write; kw...) =
    apply!(copy_simulation(sim), f, call, read, write; kw...)

"""
    step = prepare_apply(sim, transition::Symbol, call, read, write;
                         add_existing, with_edge, params)
    step()   # apply!(sim, transition, call, read, write; ...)

One apply! prepared once and run by calling the result (vg_apply_prepare,
vg_apply_call_run): the same vg_apply call with its arguments converted and
copied once, for loops whose per-call argument handling costs more than a
small simulation's step.  The transition name is checked when the call is
prepared, everything else at each run.
"""
mutable struct PreparedApply
    h::Ptr{Cvoid}
    sim::Simulation
end
function prepare_apply(sim::Simulation, f::Symbol, call, read, write;
                       add_existing = [], with_edge = nothing, params = Float64[])
    c, r, w, a = refs(sim, call), refs(sim, read), refs(sim, write), refs(sim, add_existing)
    we = with_edge === nothing ? Cint(-1) : Cint(sim.model.edges[with_edge])
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:vg_apply_prepare, LIB), Cint,
                (Ptr{Cvoid}, Cstring, Ptr{Cint}, Cint, Ptr{Cint}, Cint, Ptr{Cint}, Cint,
                 Ptr{Cint}, Cint, Cint, Ptr{Cdouble}, Cint, Ptr{Ptr{Cvoid}}),
                sim.h, String(f), c, length(c), r, length(r), w, length(w), a, length(a), we,
                Float64.(params), length(params), h))
    finalizer(release!, PreparedApply(h[], sim))
end
"release!(step) frees a prepared apply! (it keeps no device memory)"
function release!(p::PreparedApply)
    p.h == C_NULL || ccall((:vg_apply_call_destroy, LIB), Cint, (Ptr{Cvoid},), p.h)
    p.h = C_NULL
    nothing
end
function (p::PreparedApply)()
    p.h == C_NULL && error("this prepared apply! was released")
    p.sim.h == C_NULL && error("the simulation of this prepared apply! is finished")
    check(ccall((:vg_apply_call_run, LIB), Cint, (Ptr{Cvoid},), p.h))
    p.sim
end

"""
    apply_host!(sim, transition::Symbol, call, read, write, T, states::Vector{T};
                add_existing, with_edge, params)

apply! for agent vectors kept in host memory: `states` (the agents of type
T in index order) are uploaded, the transition runs, and the new states are
returned as a Vector{T} (vg_apply_host; the download of finished rows
overlaps the gather kernel of bounded_confidence).
"""
function apply_host!(sim::Simulation, f::Symbol, call, read, write, ::Type{T}, states::Vector{T};
                     add_existing = [], with_edge = nothing, params = Float64[]) where T
    c, r, w, a = refs(sim, call), refs(sim, read), refs(sim, write), refs(sim, add_existing)
    we = with_edge === nothing ? Cint(-1) : Cint(sim.model.edges[with_edge])
    n = length(states)
    cin = [ft[getfield(s, i) for s in states] for (i, ft) in enumerate(fieldtypes(T))]
    cout = [Vector{ft}(undef, n) for ft in fieldtypes(T)]
    pin = Ptr{Cvoid}[pointer(x) for x in cin]
    pout = Ptr{Cvoid}[pointer(x) for x in cout]
    GC.@preserve cin cout check(ccall((:vg_apply_host, LIB), Cint,
                (Ptr{Cvoid}, Cstring, Ptr{Cint}, Cint, Ptr{Cint}, Cint, Ptr{Cint}, Cint,
                 Ptr{Cint}, Cint, Cint, Ptr{Cdouble}, Cint, Cint, Ptr{Ptr{Cvoid}},
                 Ptr{Ptr{Cvoid}}, UInt64),
                sim.h, String(f), c, length(c), r, length(r), w, length(w), a, length(a), we,
                Float64.(params), length(params), sim.model.agents[T], pin, pout, n))
    fromcolumns(T, cout, n)
end

transition_names() =
    Symbol.(split(unsafe_string(ccall((:vg_transition_names, LIB), Cstring, ())), ","))

"""
    mapreduce(sim, field::Symbol, op, T; init, datatype)

mapreduce -- src/AgentMethods.jl:533-565, src/EdgeMethods.jl:972-1001, with
`f` a field projection (the library reduces on the device).
"""
function mapreduce(sim::Simulation, field::Symbol, op, ::Type{T};
                   init = nothing, datatype = nothing) where T
    isedge = haskey(sim.model.edges, T)
    fi = findfirst(==(field), fieldnames(T)) - 1
    FT = fieldtype(T, field)
    out_dt = FT <: AbstractFloat ? 11 : (FT === Bool && op in (&, |, max, min)) ? 1 : 9
    out = Ref{UInt64}(0)
    fn = isedge ? :vg_mapreduce_edges : :vg_mapreduce_agents
    idx = isedge ? sim.model.edges[T] : sim.model.agents[T]
    check(ccall((fn, LIB), Cint,
                (Ptr{Cvoid}, Cint, Cint, Cint, Cdouble, Cint, Cint, Cint, Cdouble, Ptr{Cvoid}),
                sim.h, idx, fi, 0, 0.0, OPS[op], out_dt, init !== nothing,
                init === nothing ? 0.0 : Float64(init), out))
    out_dt == 11 ? reinterpret(Float64, out[]) : out_dt == 1 ? out[] != 0 :
                   reinterpret(Int64, out[])
end

function fromcolumns(::Type{T}, cols, n) where T
    [T((cols[f][i] for f in 1:fieldcount(T))...) for i in 1:n]
end

"agentstate(sim, id, T) -- src/AgentMethods.jl:91-154"
function agentstate(sim::Simulation, id::AgentID, ::Type{T}) where T
    cols = [Vector{ft}(undef, 1) for ft in fieldtypes(T)]
    ptrs = Ptr{Cvoid}[pointer(c) for c in cols]
    GC.@preserve cols check(ccall((:vg_agentstate, LIB), Cint,
        (Ptr{Cvoid}, UInt64, Cint, Ptr{Ptr{Cvoid}}), sim.h, id, sim.model.agents[T], ptrs))
    fromcolumns(T, cols, 1)[1]
end

function agentstate_flexible(sim::Simulation, id::AgentID)
    tnr = Int(id >> 56)
    T = first(k for (k, v) in sim.model.agents if v == tnr)
    agentstate(sim, id, T)
end

function rowcall(sim, fn, id, ::Type{T}) where T
    n = Ref{Int64}(0)
    e = sim.model.edges[T]
    if fn === :vg_neighborids
        check(ccall((fn, LIB), Cint, (Ptr{Cvoid}, UInt64, Cint, Ptr{UInt64}, UInt64, Ptr{Int64}),
                    sim.h, id, e, C_NULL, 0, n))
    else
        check(ccall((fn, LIB), Cint, (Ptr{Cvoid}, UInt64, Cint, Ptr{Cvoid}, Ptr{Cvoid}, UInt64,
                                      Ptr{Int64}), sim.h, id, e, C_NULL, C_NULL, 0, n))
    end
    n[]
end

"edges(sim, id, T) -- src/EdgeMethods.jl:705-715"
function edges(sim::Simulation, id::AgentID, ::Type{T}) where T
    n = Ref{Int64}(0)
    e = sim.model.edges[T]
    check(ccall((:vg_edges, LIB), Cint,
                (Ptr{Cvoid}, UInt64, Cint, Ptr{UInt64}, Ptr{Ptr{Cvoid}}, UInt64, Ptr{Int64}),
                sim.h, id, e, C_NULL, C_NULL, 0, n))
    n[] < 0 && return nothing
    from = Vector{AgentID}(undef, n[])
    cols = [Vector{ft}(undef, n[]) for ft in fieldtypes(T)]
    ptrs = Ptr{Cvoid}[pointer(c) for c in cols]
    GC.@preserve cols check(ccall((:vg_edges, LIB), Cint,
        (Ptr{Cvoid}, UInt64, Cint, Ptr{UInt64}, Ptr{Ptr{Cvoid}}, UInt64, Ptr{Int64}),
        sim.h, id, e, from, ptrs, n[], n))
    [Edge(from[i], fromcolumns(T, cols, n[])[i]) for i in 1:n[]]
end

"neighborids(sim, id, T) -- src/EdgeMethods.jl:718-742"
function neighborids(sim::Simulation, id::AgentID, ::Type{T}) where T
    n = Ref{Int64}(0)
    e = sim.model.edges[T]
    check(ccall((:vg_neighborids, LIB), Cint,
                (Ptr{Cvoid}, UInt64, Cint, Ptr{UInt64}, UInt64, Ptr{Int64}),
                sim.h, id, e, C_NULL, 0, n))
    n[] < 0 && return nothing
    out = Vector{AgentID}(undef, n[])
    check(ccall((:vg_neighborids, LIB), Cint,
                (Ptr{Cvoid}, UInt64, Cint, Ptr{UInt64}, UInt64, Ptr{Int64}),
                sim.h, id, e, out, n[], n))
    out
end

neighborstates(sim::Simulation, id::AgentID, ::Type{E}, ::Type{A}) where {E, A} =
    (ids = neighborids(sim, id, E); ids === nothing ? nothing : [agentstate(sim, i, A) for i in ids])

"the normalised hint bits of edge type T (vg_model_edge_hints)"
function edgehints(model::ModelTypes, ::Type{T}) where T
    h = Ref{Cuint}(0)
    check(ccall((:vg_model_edge_hints, LIB), Cint, (Ptr{Cvoid}, Cint, Ptr{Cuint}),
                model.h, model.edges[T], h))
    h[]
end

function notdefined(sim, ::Type{T}, fn, hints...) where T
    h = edgehints(sim.model, T)
    any(x -> h & HINTS[x] != 0, hints) &&
        throw(AssertionError("$fn is not defined for edgetypes with the " *
                             join(string.(":", hints), " or ") * " hint"))
end

"neighborstates_flexible(sim, id, T) -- src/Edge.jl:303-306"
neighborstates_flexible(sim::Simulation, id::AgentID, ::Type{E}) where E =
    (ids = neighborids(sim, id, E); ids === nothing ? nothing : [agentstate_flexible(sim, i) for i in ids])

"neighborids_iter(sim, id, T) -- src/EdgeMethods.jl:744-760"
neighborids_iter(sim::Simulation, id::AgentID, ::Type{E}) where E =
    (notdefined(sim, E, "neighborids_iter", :SingleEdge, :IgnoreFrom);
     ids = neighborids(sim, id, E); ids === nothing ? nothing : (i for i in ids))

"edgestates_iter(sim, id, T) -- src/Edge.jl:208-224"
edgestates_iter(sim::Simulation, id::AgentID, ::Type{E}) where E =
    (notdefined(sim, E, "edgestates_iter", :SingleEdge, :Stateless);
     es = edgestates(sim, id, E); es === nothing ? nothing : (e for e in es))

"neighborstates_iter(sim, id, T, A) -- src/EdgeMethods.jl:783-803"
neighborstates_iter(sim::Simulation, id::AgentID, ::Type{E}, ::Type{A}) where {E, A} =
    (notdefined(sim, E, "neighborstates_iter", :SingleEdge, :IgnoreFrom);
     ids = neighborids(sim, id, E); ids === nothing ? nothing : (agentstate(sim, i, A) for i in ids))

"neighborstates_flexible_iter(sim, id, T) -- src/Edge.jl:328-335"
neighborstates_flexible_iter(sim::Simulation, id::AgentID, ::Type{E}) where E =
    (ids = neighborids(sim, id, E); ids === nothing ? nothing : (agentstate_flexible(sim, i) for i in ids))

"edgestates(sim, id, T) -- src/EdgeMethods.jl:805-829"
function edgestates(sim::Simulation, id::AgentID, ::Type{T}) where T
    es = edges(sim, id, T)
    es === nothing ? nothing : [e.state for e in es]
end

"num_edges(sim, id, T) -- src/EdgeMethods.jl:851-869"
function num_edges(sim::Simulation, id::AgentID, ::Type{T}) where T
    n = Ref{Int64}(0)
    check(ccall((:vg_num_edges, LIB), Cint, (Ptr{Cvoid}, UInt64, Cint, Ptr{Int64}),
                sim.h, id, sim.model.edges[T], n))
    n[]
end

"num_edges(sim, T; write) -- src/Edge.jl:373-389"
function num_edges(sim::Simulation, ::Type{T}; write = false) where T
    n = Ref{UInt64}(0)
    check(ccall((:vg_num_edges_total, LIB), Cint, (Ptr{Cvoid}, Cint, Cint, Ptr{UInt64}),
                sim.h, sim.model.edges[T], write, n))
    Int(n[])
end

"has_edge(sim, id, T) -- src/EdgeMethods.jl:873-892"
function has_edge(sim::Simulation, id::AgentID, ::Type{T}) where T
    n = Ref{Cint}(0)
    check(ccall((:vg_has_edge, LIB), Cint, (Ptr{Cvoid}, UInt64, Cint, Ptr{Cint}),
                sim.h, id, sim.model.edges[T], n))
    n[] != 0
end

"num_agents(sim, T) -- src/Agent.jl:324-343"
function num_agents(sim::Simulation, ::Type{T}) where T
    n = Ref{UInt64}(0)
    check(ccall((:vg_num_agents, LIB), Cint, (Ptr{Cvoid}, Cint, Ptr{UInt64}),
                sim.h, sim.model.agents[T], n))
    Int(n[])
end

function all_with_ids(sim::Simulation, ::Type{T}) where T
    n = Ref{UInt64}(0)
    tnr = sim.model.agents[T]
    check(ccall((:vg_all_agents, LIB), Cint,
                (Ptr{Cvoid}, Cint, Ptr{Ptr{Cvoid}}, Ptr{UInt64}, UInt64, Ptr{UInt64}),
                sim.h, tnr, C_NULL, C_NULL, 0, n))
    cols = [Vector{ft}(undef, n[]) for ft in fieldtypes(T)]
    ptrs = Ptr{Cvoid}[pointer(c) for c in cols]
    ids = Vector{AgentID}(undef, n[])
    GC.@preserve cols check(ccall((:vg_all_agents, LIB), Cint,
        (Ptr{Cvoid}, Cint, Ptr{Ptr{Cvoid}}, Ptr{UInt64}, UInt64, Ptr{UInt64}),
        sim.h, tnr, ptrs, ids, n[], n))
    fromcolumns(T, cols, n[]), ids
end
"all_agents(sim, T) -- src/Agent.jl:234-260"
all_agents(sim::Simulation, ::Type{T}) where T = all_with_ids(sim, T)[1]
"all_agentids(sim, T) -- src/Agent.jl:287-313"
all_agentids(sim::Simulation, ::Type{T}) where T = all_with_ids(sim, T)[2]

"add_raster!(sim, name, dims, constructor) -- src/Raster.jl:32-54"
function add_raster!(sim::Simulation, name::Symbol, dims::NTuple{N, Int}, ctor) where N
    cells = [ctor(pos) for pos in CartesianIndices(dims)]
    T = eltype(cells)
    cols = columns(vec(cells))
    ptrs = Ptr{Cvoid}[pointer(c) for c in cols]
    ids = Vector{AgentID}(undef, length(cells))
    GC.@preserve cols check(ccall((:vg_add_raster, LIB), Cint,
        (Ptr{Cvoid}, Cstring, Cint, Ptr{Int64}, Cint, Ptr{Ptr{Cvoid}}, Ptr{UInt64}),
        sim.h, String(name), N, collect(Int64, dims), sim.model.agents[T], ptrs, ids))
    sim.rasters[name] = dims
    reshape(ids, dims)
end

const METRICS = Dict(:chebyshev => 0, :euclidean => 1, :manhatten => 2)

"connect_raster_neighbors!(sim, name, ctor; distance, metric, periodic) -- src/Raster.jl:139-167"
function connect_raster_neighbors!(sim::Simulation, name::Symbol, state::T;
                                   distance = 1, metric = :chebyshev, periodic = true,
                                   implicit = false) where T
    cols = columns([state])
    ptrs = Ptr{Cvoid}[pointer(c) for c in cols]
    GC.@preserve cols check(ccall((:vg_connect_raster_neighbors, LIB), Cint,
        (Ptr{Cvoid}, Cstring, Cint, Ptr{Ptr{Cvoid}}, Cdouble, Cint, Cint, Cint),
        sim.h, String(name), sim.model.edges[T], isempty(ptrs) ? C_NULL : ptrs,
        distance, METRICS[metric], periodic, implicit))
end

"move_to!(sim, name, id, pos, edge_from_raster, edge_to_raster; ...) -- src/Raster.jl:437-477"
function move_to!(sim::Simulation, name::Symbol, id::AgentID, pos, from_state, to_state;
                  distance = 0, metric = :chebyshev, periodic = true, only_surrounding = false)
    ef = from_state === nothing ? Cint(-1) : Cint(sim.model.edges[typeof(from_state)])
    et = to_state === nothing ? Cint(-1) : Cint(sim.model.edges[typeof(to_state)])
    cf = from_state === nothing ? [] : columns([from_state])
    ct = to_state === nothing ? [] : columns([to_state])
    pf = Ptr{Cvoid}[pointer(c) for c in cf]
    pt = Ptr{Cvoid}[pointer(c) for c in ct]
    GC.@preserve cf ct check(ccall((:vg_move_to, LIB), Cint,
        (Ptr{Cvoid}, Cstring, UInt64, Ptr{Int64}, Cint, Ptr{Ptr{Cvoid}}, Cint, Ptr{Ptr{Cvoid}},
         Cdouble, Cint, Cint, Cint),
        sim.h, String(name), id, collect(Int64, Tuple(pos)), ef, isempty(pf) ? C_NULL : pf,
        et, isempty(pt) ? C_NULL : pt, distance, METRICS[metric], periodic, only_surrounding))
end

"cellid(sim, name, pos) -- src/Raster.jl:403-405"
function cellid(sim::Simulation, name::Symbol, pos)
    out = Ref{UInt64}(0)
    check(ccall((:vg_cellid, LIB), Cint, (Ptr{Cvoid}, Cstring, Ptr{Int64}, Ptr{UInt64}),
                sim.h, String(name), collect(Int64, Tuple(pos)), out))
    out[]
end

"rastervalues(sim, name, field) -- src/Raster.jl:353-387"
function raster_dims(sim::Simulation, name::Symbol)
    get!(sim.rasters, name) do  # a simulation read from a snapshot knows no names yet
        d = zeros(Int64, 4)
        nd = Ref{Cint}(0)
        check(ccall((:vg_raster_dims, LIB), Cint, (Ptr{Cvoid}, Cstring, Ptr{Int64}, Ptr{Cint}),
                    sim.h, String(name), d, nd))
        Tuple(d[1:nd[]])
    end
end

function rastervalues(sim::Simulation, name::Symbol, field::Symbol)
    dims = raster_dims(sim, name)
    T = agentstate_type(sim, cellid(sim, name, ntuple(_ -> 1, length(dims))))
    FT = fieldtype(T, field)
    out = Vector{FT}(undef, prod(dims))
    check(ccall((:vg_rastervalues, LIB), Cint, (Ptr{Cvoid}, Cstring, Cint, Ptr{Cvoid}),
                sim.h, String(name), findfirst(==(field), fieldnames(T)) - 1, out))
    reshape(out, dims)
end
agentstate_type(sim, id) = first(k for (k, v) in sim.model.agents if v == Int(id >> 56))
calc_rasterstate(sim::Simulation, name::Symbol, field::Symbol) = rastervalues(sim, name, field)

param(sim::Simulation, name::Symbol) =
    (v = Ref{Cdouble}(0); check(ccall((:vg_param, LIB), Cint, (Ptr{Cvoid}, Cstring, Ptr{Cdouble}),
                                      sim.h, String(name), v)); v[])
set_param!(sim::Simulation, name::Symbol, v) =
    check(ccall((:vg_set_param, LIB), Cint, (Ptr{Cvoid}, Cstring, Cdouble), sim.h, String(name), v))
get_global(sim::Simulation, name::Symbol) =
    (v = Ref{Cdouble}(0); check(ccall((:vg_get_global, LIB), Cint,
                                      (Ptr{Cvoid}, Cstring, Ptr{Cdouble}), sim.h, String(name), v)); v[])
set_global!(sim::Simulation, name::Symbol, v) =
    check(ccall((:vg_set_global, LIB), Cint, (Ptr{Cvoid}, Cstring, Cdouble), sim.h, String(name), v))

"""
    bind_param!(sim, transition::Symbol, slot, name::Symbol; kind = :global)

Parameter `slot` (0-based) of every later apply! of `transition` takes the
current value of the global (or, kind = :param, the param) `name`: the
kernel reads get_global(sim, name) / param(sim, name) at each step.
"""
bind_param!(sim::Simulation, f::Symbol, slot::Integer, name::Symbol; kind = :global) =
    check(ccall((:vg_bind_param, LIB), Cint, (Ptr{Cvoid}, Cstring, Cint, Cint, Cstring),
                sim.h, String(f), slot, kind === :param ? 0 : 1, String(name)))
push_global!(sim::Simulation, name::Symbol, v) =
    check(ccall((:vg_push_global, LIB), Cint, (Ptr{Cvoid}, Cstring, Cdouble), sim.h, String(name), v))

"""
    add_graph!(sim, nv, edges, agent_constructor, edge_constructor; directed)

add_graph! -- src/GraphsSupport.jl:34-57, with the graph given as its vertex
count and its edge list `(src, dst)` in the graph's edge order (so that no
Graphs.jl import is needed).  Returns the new agents' ids.
"""
function add_graph!(sim::Simulation, nv::Integer, edges::Vector{Tuple{Int,Int}},
                    agent_constructor, edge_constructor; directed::Bool = true)
    agents = [agent_constructor(v) for v in 1:nv]
    states = [edge_constructor(e) for e in edges]
    T = eltype(agents)
    acols = columns(agents)
    aptrs = Ptr{Cvoid}[pointer(c) for c in acols]
    E = eltype(states)
    ecols = columns(states)
    eptrs = Ptr{Cvoid}[pointer(c) for c in ecols]
    src = UInt64[e[1] for e in edges]
    dst = UInt64[e[2] for e in edges]
    ids = Vector{AgentID}(undef, nv)
    GC.@preserve acols ecols check(ccall((:vg_add_graph, LIB), Cint,
        (Ptr{Cvoid}, Cint, UInt64, Ptr{Ptr{Cvoid}}, Cint, UInt64, Ptr{UInt64}, Ptr{UInt64},
         Cint, Ptr{Ptr{Cvoid}}, Ptr{UInt64}),
        sim.h, sim.model.agents[T], nv, aptrs, sim.model.edges[E], length(edges), src, dst,
        directed ? 1 : 0, isempty(eptrs) ? C_NULL : eptrs, ids))
    ids
end

"remove_edges!(sim, to, T) / remove_edges!(sim, from, to, T) -- src/EdgeMethods.jl:527-599"
remove_edges!(sim::Simulation, to::AgentID, ::Type{T}) where T =
    check(ccall((:vg_remove_edges, LIB), Cint,
                (Ptr{Cvoid}, Cint, UInt64, Ptr{UInt64}, Ptr{UInt64}),
                sim.h, sim.model.edges[T], 1, C_NULL, [to]))
remove_edges!(sim::Simulation, from::AgentID, to::AgentID, ::Type{T}) where T =
    check(ccall((:vg_remove_edges, LIB), Cint,
                (Ptr{Cvoid}, Cint, UInt64, Ptr{UInt64}, Ptr{UInt64}),
                sim.h, sim.model.edges[T], 1, [from], [to]))

"add_agent_per_process!(sim, agent) -- src/Agent.jl:367-388"
function add_agent_per_process!(sim::Simulation, agent::T) where T
    cols = columns([agent])
    ptrs = Ptr{Cvoid}[pointer(c) for c in cols]
    id = Ref{UInt64}(0)
    GC.@preserve cols check(ccall((:vg_add_agent_per_process, LIB), Cint,
        (Ptr{Cvoid}, Cint, Ptr{Ptr{Cvoid}}, Ptr{UInt64}), sim.h, sim.model.agents[T], ptrs, id))
    id[]
end

"""
    write_snapshot(sim, path) / read_snapshot(model, path)

The role of write_snapshot / read_snapshot! (src/HDF5.jl:688-715,
1594-1660) in the library's own checkpoint format (not HDF5).
"""
write_snapshot(sim::Simulation, path::AbstractString) =
    check(ccall((:vg_sim_save, LIB), Cint, (Ptr{Cvoid}, Cstring), sim.h, path))
function read_snapshot(model::ModelTypes, path::AbstractString; stream = C_NULL)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:vg_sim_load, LIB), Cint, (Ptr{Cvoid}, Cstring, Ptr{Cvoid}, Ptr{Ptr{Cvoid}}),
                model.h, path, stream, h))
    sim = Simulation(h[], model, Dict{Symbol, Tuple}())
    finalizer(s -> s.h == C_NULL || ccall((:vg_sim_destroy, LIB), Cint, (Ptr{Cvoid},), s.h), sim)
    sim
end

end # module
