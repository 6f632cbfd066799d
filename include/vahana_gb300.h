/*
 * vahana_gb300.h -- C ABI of the GB300-native Vahana.jl transition step.
 *
 * One shared library (libvahana_gb300.so) owns every device buffer of a
 * simulation: agent state as struct-of-arrays read/write double buffers,
 * and each edge type as a CSR keyed by target agent, kept in the
 * reference's edge-insertion order.  Transition functions are bound by
 * name to hand-written sm_103a kernels.  The signatures below are what a
 * Julia `ccall` (or Python ctypes) binding of Vahana's public API calls;
 * each entry cites the reference function it replaces (paths are relative
 * to the Vahana.jl v1.4.7 source tree).
 *
 * Conventions
 *   - Every function returns an int status: VG_OK (0) or a VG_ERR_* code.
 *     VG_ERR_ASSERT marks the cases where the reference raises an
 *     AssertionError; a binding rethrows it as AssertionError.
 *     vg_last_error() returns the message of the last failure of the
 *     calling thread.
 *   - Agent IDs keep the reference's bit layout (src/Agent.jl:30-115):
 *     type_nr << 56 | process << 36 | agent_nr, with process = 0 (one GPU,
 *     no MPI ranks) and agent_nr 1-based.
 *   - A "type reference" (used in call/read/write/add_existing lists) is
 *     an agent type number (1..255) or VG_EDGE(edge_type_index).
 *   - Host pointers are plain host memory; nothing here takes a torch type.
 *   - All device work of a simulation runs on one CUDA stream (given at
 *     vg_sim_create, or the library's own); calls on one handle are not
 *     re-entrant (the reference is single threaded, src/MPIinit.jl:22).
 */
#ifndef VAHANA_GB300_H
#define VAHANA_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define VG_OK 0
#define VG_ERR_ASSERT 1   /* reference raises AssertionError                */
#define VG_ERR_ARG 2      /* malformed argument (unknown name, bad pointer) */
#define VG_ERR_CUDA 3     /* CUDA runtime error                             */
#define VG_ERR_NOMEM 4    /* device allocation failed / over a stated limit */
#define VG_ERR_DEVICE 5   /* a kernel reported an error through its status  */
#define VG_ERR_STATE 6    /* call not allowed in the current phase          */

/* ---- field data types (SoA columns of agent and edge state) ----------- */
#define VG_BOOL 1
#define VG_U8 2
#define VG_I8 3
#define VG_U16 4
#define VG_I16 5
#define VG_U32 6
#define VG_I32 7
#define VG_U64 8
#define VG_I64 9
#define VG_F32 10
#define VG_F64 11

/* ---- hints (src/ModelTypes.jl:81-230) ---------------------------------- */
#define VG_HINT_IMMORTAL 0x01u          /* agent  :Immortal                 */
#define VG_HINT_INDEPENDENT 0x02u       /* agent  :Independent              */
#define VG_HINT_STATELESS 0x10u         /* edge   :Stateless                */
#define VG_HINT_IGNOREFROM 0x20u        /* edge   :IgnoreFrom               */
#define VG_HINT_SINGLETYPE 0x40u        /* edge   :SingleType (target=...)  */
#define VG_HINT_SINGLEEDGE 0x80u        /* edge   :SingleEdge               */
#define VG_HINT_IGNORESOURCESTATE 0x100u /* edge  :IgnoreSourceState        */
#define VG_HINT_NUMEDGESONLY 0x200u     /* edge   :NumEdgesOnly             */
#define VG_HINT_HASEDGEONLY 0x400u      /* edge   :HasEdgeOnly              */

/* ---- type references in call/read/write lists -------------------------- */
#define VG_EDGE(e) (0x10000 | (e))

/* ---- reduction operators of mapreduce (src/Helpers.jl:44-81) ----------- */
#define VG_OP_ADD 1
#define VG_OP_MUL 2
#define VG_OP_MAX 3
#define VG_OP_MIN 4
#define VG_OP_AND 5
#define VG_OP_OR 6
/* or-ed into op: the fold order.  By default Float + and * fold
 * sequentially in the reference's order (bit-identical results) and every
 * other reduction, whose result does not depend on the order, takes a
 * parallel tree.  VG_REDUCE_ORDERED forces the sequential fold,
 * VG_REDUCE_TREE the tree (Float + and *: within 2 (n - 1) 2^-53 sum|f(x)|
 * of the sequential result). */
#define VG_REDUCE_ORDERED 0x100
#define VG_REDUCE_TREE 0x200

/* map function applied to each element before the reduction (mapreduce's
 * `f`): the field itself, or the field compared with a constant. */
#define VG_MAP_FIELD 0
#define VG_MAP_EQ 1
#define VG_MAP_NE 2
#define VG_MAP_LT 3
#define VG_MAP_GT 4

/* raster metrics (src/Raster.jl:82-96) */
#define VG_METRIC_CHEBYSHEV 0
#define VG_METRIC_EUCLIDEAN 1
#define VG_METRIC_MANHATTEN 2

typedef struct vg_model vg_model;
typedef struct vg_sim vg_sim;

/* ---- library ----------------------------------------------------------- */
const char *vg_last_error(void);
int vg_version(void);
/* Number of CUDA devices visible (0 here means: no GPU; every compute call
 * will fail with VG_ERR_CUDA, there is no CPU fallback). */
int vg_device_count(int *out);

/* ---- model registry ---------------------------------------------------- */
/* ModelTypes() -- src/ModelTypes.jl:32-41 */
int vg_model_create(vg_model **out);
void vg_model_destroy(vg_model *m);
/* register_agenttype!(types, T, hints...) -- src/ModelTypes.jl:81-106.
 * Fields are the struct's fields in declaration order. *type_nr_out is the
 * 1-based type number used in AgentIDs. */
int vg_model_register_agenttype(vg_model *m, const char *name, int nfields,
                                const char *const *field_names,
                                const int *field_dtypes, unsigned hints,
                                int *type_nr_out);
/* register_edgetype!(types, T, hints...; target, size) --
 * src/ModelTypes.jl:158-230.  target_type_nr is 0 unless :SingleType;
 * size is the optional `size` keyword (0 = not given). */
int vg_model_register_edgetype(vg_model *m, const char *name, int nfields,
                               const char *const *field_names,
                               const int *field_dtypes, unsigned hints,
                               int target_type_nr, int64_t size,
                               int *edge_type_out);
/* register_param! / register_global! -- scalar f64 values by name. */
int vg_model_register_param(vg_model *m, const char *name, double dflt);
int vg_model_register_global(vg_model *m, const char *name, double dflt);
/* create_model(types, name) -- src/Simulation.jl:115-207 */
int vg_model_finalize(vg_model *m, const char *name);
/* has_hint(sim, T, hint) -- src/ModelTypes.jl:235-242; returns the effective
 * (normalised) hint bits of an edge type. */
int vg_model_edge_hints(const vg_model *m, int edge_type, unsigned *out);
int vg_model_type_by_name(const vg_model *m, const char *name, int *out);

/* ---- simulation lifecycle ---------------------------------------------- */
/* create_simulation(model, params, globals; name) -- src/Simulation.jl:261-339.
 * stream is a cudaStream_t (NULL = the library creates its own). */
int vg_sim_create(vg_model *m, const char *name, void *stream, vg_sim **out);
/* finish_simulation! -- src/Simulation.jl:551-573 */
int vg_sim_destroy(vg_sim *s);
/* copy_simulation(sim) -- src/Simulation.jl:500-510 */
int vg_sim_copy(vg_sim *s, vg_sim **out);
/* finish_init!(sim) -- src/Simulation.jl:403-476 (one process: no
 * partitioning, ids stay as issued). Uploads the staged graph and builds the
 * device CSR of every edge type in insertion order. */
int vg_finish_init(vg_sim *s);
int vg_sim_num_transitions(vg_sim *s, int64_t *out);
int vg_sim_set_stream(vg_sim *s, void *stream);
/* Waits for the simulation's stream and reports a kernel status word set
 * by an asynchronous apply! (as the AssertionError apply! would raise). */
int vg_sim_synchronize(vg_sim *s);
/* async != 0: apply! returns without waiting for the device; errors that
 * kernels report surface at the next synchronizing call (vg_sim_synchronize,
 * a read back, or switching async off).  Default off: every apply! checks. */
int vg_sim_set_async(vg_sim *s, int async);
/* Overwrite the first n agents' state of a type from host SoA columns
 * between transitions (fields[i] may be NULL to keep a column).  No direct
 * reference counterpart: it is how a host binding pushes a state array it
 * changed back into a device-resident simulation. */
int vg_write_agents(vg_sim *s, int type_nr, const void *const *fields,
                    uint64_t n);
/* Bytes of device memory the simulation holds (admission by footprint). */
int vg_sim_device_bytes(vg_sim *s, uint64_t *out);
/* disable_transition_checks(sim, disable) -- src/Helpers.jl:259-262 */
int vg_disable_transition_checks(vg_sim *s, int disable);

/* ---- params and globals (src/Simulation.jl:587-630, src/Global.jl) ----- */
int vg_set_param(vg_sim *s, const char *name, double v);
int vg_param(vg_sim *s, const char *name, double *out);
int vg_set_global(vg_sim *s, const char *name, double v);
int vg_get_global(vg_sim *s, const char *name, double *out);
/* Binds parameter slot `slot` of the named transition to this simulation's
 * param (kind 0) or global (kind 1) `name`: every later apply! of that
 * transition passes the current value in that slot, so a transition reads
 * param(sim, name) / get_global(sim, name) (src/Simulation.jl:587,
 * src/Global.jl:10) and set_global! between steps reaches the kernels.
 * apply! must still pass at least slot + 1 parameters (the bound slot's
 * value is replaced).  vg_unbind_params(s, NULL) removes every binding. */
int vg_bind_param(vg_sim *s, const char *transition, int slot, int kind, const char *name);
int vg_unbind_params(vg_sim *s, const char *transition);
int vg_push_global(vg_sim *s, const char *name, double v);
int vg_global_series(vg_sim *s, const char *name, double *out, uint64_t cap,
                     uint64_t *n_out);

/* Checkpoint / restore of an initialized simulation (the reference's
 * write_snapshot / read_snapshot!, src/HDF5.jl:688-715, 1594-1660, write
 * HDF5; this is the library's own binary format, no HDF5 library is used).
 * The file holds every agent type's read state, died flags, reuse stack
 * and nextid, every edge type's CSR (or implicit stencil), rasters, params,
 * globals and num_transitions, with a fingerprint of the model: loading
 * into a different model fails with VG_ERR_ASSERT.  A loaded simulation
 * continues bit-identically to the saved one. */
int vg_sim_save(vg_sim *s, const char *path);
int vg_sim_load(vg_model *m, const char *path, void *stream, vg_sim **out);

/* ---- agents ------------------------------------------------------------ */
/* add_agents!(sim, agents) / add_agent! -- src/Agent.jl:174-180,
 * src/AgentMethods.jl:65-89.  fields[i] points to n values of field i
 * (SoA, the field's dtype).  Before finish_init! only, or through
 * vg_add_agent_per_process after it (src/Agent.jl:367-388). */
int vg_add_agents(vg_sim *s, int type_nr, uint64_t n,
                  const void *const *fields, uint64_t *ids_out);
int vg_add_agent_per_process(vg_sim *s, int type_nr,
                             const void *const *fields, uint64_t *id_out);
/* agentstate(sim, id, T) -- src/AgentMethods.jl:91-154 (host read back) */
int vg_agentstate(vg_sim *s, uint64_t id, int type_nr, void *const *fields_out);
/* num_agents(sim, T) -- src/Agent.jl:324-343 */
int vg_num_agents(vg_sim *s, int type_nr, uint64_t *out);
/* Slot count (nextid - 1): the length of the state vectors. */
int vg_agent_slots(vg_sim *s, int type_nr, uint64_t *out);
/* all_agents / all_agentids -- src/Agent.jl:234-313.  Writes the living
 * agents in index order; call with cap = 0 to get the count. */
int vg_all_agents(vg_sim *s, int type_nr, void *const *fields_out,
                  uint64_t *ids_out, uint64_t cap, uint64_t *n_out);
/* Bulk read of all slots (living and died) of the read buffers; died_out
 * may be NULL.  Used for parity checks of whole states. */
int vg_read_agents(vg_sim *s, int type_nr, void *const *fields_out,
                   uint8_t *died_out, uint64_t cap, uint64_t *n_out);
/* Device pointer of a field's read buffer (for zero-copy consumers). */
int vg_agent_field_device_ptr(vg_sim *s, int type_nr, int field, void **out);

/* ---- edges ------------------------------------------------------------- */
/* add_edge!(sim, from, to, state) / add_edges! -- src/EdgeMethods.jl:388-523,
 * src/Edge.jl:81-96.  Before finish_init!, or between transitions when
 * transition checks are disabled (as the reference's tests do).
 * payload[i] points to n values of edge field i (may be NULL for stateless
 * types).  Edges are appended in array order. */
int vg_add_edges(vg_sim *s, int edge_type, uint64_t n, const uint64_t *from,
                 const uint64_t *to, const void *const *payload);
/* add_graph!(sim, graph, agent_constructor, edge_constructor) --
 * src/GraphsSupport.jl:34-57, before finish_init!.  The graph's nv vertices
 * become agents of type_nr (fields: nv values per field, vertex order);
 * its ne edges, in the graph's edge order as 1-based vertex numbers
 * src[k] -> dst[k] with payload columns of ne values, are added as
 * add_edge!(agent[src], agent[dst]) and, when directed == 0, then
 * add_edge!(agent[dst], agent[src]) with the same state.  ids_out (nv
 * entries, may be NULL) receives the agents' ids. */
int vg_add_graph(vg_sim *s, int type_nr, uint64_t nv, const void *const *fields,
                 int edge_type, uint64_t ne, const uint64_t *src, const uint64_t *dst,
                 int directed, const void *const *payload, uint64_t *ids_out);
/* remove_edges!(sim, to, T) and remove_edges!(sim, from, to, T) --
 * src/EdgeMethods.jl:527-599.  from may be NULL (remove all edges to `to`). */
int vg_remove_edges(vg_sim *s, int edge_type, uint64_t n, const uint64_t *from,
                    const uint64_t *to);
/* Per-target accessors, read back to the host --
 * edges / neighborids / edgestates: src/EdgeMethods.jl:705-848;
 * num_edges / has_edge: :850-892.  *count_out = -1 means the reference
 * returns `nothing` (no container for this agent).  from_out / payload_out
 * may be NULL; at most cap entries are written. */
int vg_edges(vg_sim *s, uint64_t to, int edge_type, uint64_t *from_out,
             void *const *payload_out, uint64_t cap, int64_t *count_out);
int vg_neighborids(vg_sim *s, uint64_t to, int edge_type, uint64_t *from_out,
                   uint64_t cap, int64_t *count_out);
int vg_edgestates(vg_sim *s, uint64_t to, int edge_type,
                  void *const *payload_out, uint64_t cap, int64_t *count_out);
int vg_num_edges(vg_sim *s, uint64_t to, int edge_type, int64_t *out);
int vg_has_edge(vg_sim *s, uint64_t to, int edge_type, int *out);
/* num_edges(sim, T; write) -- src/Edge.jl:373-389 */
int vg_num_edges_total(vg_sim *s, int edge_type, int write, uint64_t *out);
/* Bulk read of one edge type's CSR for one target type: row_ptr (nrows+1,
 * u64), from ids (AgentIDs), payload columns.  Pass NULL to query sizes. */
int vg_read_edges(vg_sim *s, int edge_type, int target_type_nr,
                  uint64_t *row_ptr_out, uint64_t *from_out,
                  void *const *payload_out, uint64_t *nrows_out,
                  uint64_t *nedges_out);

/* ---- transitions ------------------------------------------------------- */
/* apply!(sim, f, call, read, write; add_existing, with_edge) --
 * src/Simulation.jl:720-821.  `transition` names a kernel registered in the
 * library (vg_transition_names).  Lists hold type references.  with_edge is
 * an edge type index or -1.  params/nparams are the transition's own
 * arguments (documented per transition). */
int vg_apply(vg_sim *s, const char *transition, const int *call, int ncall,
             const int *read, int nread, const int *write, int nwrite,
             const int *add_existing, int nadd, int with_edge,
             const double *params, int nparams);
/* apply! prepared once and run many times (src/Simulation.jl:720-821, the
 * same call as vg_apply): vg_apply_prepare copies the arguments of one
 * vg_apply call (the transition name is checked here, everything else at
 * each run, as vg_apply does) and vg_apply_call_run runs that call.  For a
 * binding whose foreign calls cost more than the step (a Python loop of
 * small simulations).  The handle refers to the simulation: destroy it
 * before the simulation. */
typedef struct vg_apply_call vg_apply_call;
int vg_apply_prepare(vg_sim *s, const char *transition, const int *call,
                     int ncall, const int *read, int nread, const int *write,
                     int nwrite, const int *add_existing, int nadd,
                     int with_edge, const double *params, int nparams,
                     vg_apply_call **out);
int vg_apply_call_run(vg_apply_call *c);
int vg_apply_call_destroy(vg_apply_call *c);
/* apply! for a host that keeps the called type's state in its own memory:
 * the n agents' fields of type_nr are uploaded from in_fields (host SoA
 * columns; NULL entries keep the device column), apply!(sim, transition,
 * ...) runs exactly as vg_apply, and the new state of those agents is
 * written to out_fields before the call returns -- the same result as
 * vg_write_agents, vg_apply and vg_read_agents (src/Simulation.jl:720-821
 * with the state round-tripped through the host, as a Julia caller whose
 * agent vectors live in host memory does).  For "bounded_confidence" the
 * gather launch reports each finished range of rows and the range is
 * downloaded while the launch goes on (pinned host buffers for the
 * overlap). */
int vg_apply_host(vg_sim *s, const char *transition, const int *call, int ncall,
                  const int *read, int nread, const int *write, int nwrite,
                  const int *add_existing, int nadd, int with_edge,
                  const double *params, int nparams, int type_nr,
                  const void *const *in_fields, void *const *out_fields, uint64_t n);
/* Comma-separated list of the registered transition names. */
const char *vg_transition_names(void);

/* ---- mapreduce -- src/AgentMethods.jl:533-565 (agents),
 *      src/EdgeMethods.jl:972-1001 (edges); identities from val4empty,
 *      src/Helpers.jl:44-81.  The result is written as out_dtype
 *      (VG_I64, VG_F64 or VG_BOOL).  has_init/init give the `init`
 *      keyword.  Agents fold in index order, edges in (target type, target
 *      row, insertion) order: the reference's order for agents and for
 *      :SingleType edge types (Vector containers); for the other edge types
 *      the reference iterates a Dict, whose order is not reproduced. */
int vg_mapreduce_agents(vg_sim *s, int type_nr, int field, int map_kind,
                        double map_arg, int op, int out_dtype, int has_init,
                        double init, void *out);
int vg_mapreduce_edges(vg_sim *s, int edge_type, int field, int map_kind,
                       double map_arg, int op, int out_dtype, int has_init,
                       double init, void *out);

/* ---- rasters -- src/Raster.jl ------------------------------------------- */
/* add_raster!(sim, name, dims, constructor) -- :32-54.  The cells' state is
 * given as SoA columns in column-major CartesianIndices order (first index
 * fastest); ids_out (may be NULL) receives the cell ids in that order. */
int vg_add_raster(vg_sim *s, const char *name, int ndims, const int64_t *dims,
                  int type_nr, const void *const *fields, uint64_t *ids_out);
/* connect_raster_neighbors!(sim, name, ctor; distance, metric, periodic) --
 * :139-167.  The edge constructor is a constant payload.  implicit != 0
 * keeps the edges implicit (stencil indexing, no CSR); the accessors and
 * the stencil kernels still see them in the reference's order. */
int vg_connect_raster_neighbors(vg_sim *s, const char *name, int edge_type,
                                const void *const *payload, double distance,
                                int metric, int periodic, int implicit);
/* move_to!(sim, name, id, pos, edge_from_raster, edge_to_raster; distance,
 * metric, periodic, only_surrounding) -- :437-477, in the init phase.
 * edge types may be -1 for `nothing`. */
int vg_move_to(vg_sim *s, const char *name, uint64_t id, const int64_t *pos,
               int edge_from_raster, const void *const *payload_from,
               int edge_to_raster, const void *const *payload_to,
               double distance, int metric, int periodic,
               int only_surrounding);
/* cellid(sim, name, pos) -- :403-405 (pos is 1-based) */
int vg_cellid(vg_sim *s, const char *name, const int64_t *pos, uint64_t *out);
int vg_raster_dims(vg_sim *s, const char *name, int64_t *dims_out,
                   int *ndims_out);
/* rastervalues(sim, name, field) / calc_rasterstate(sim, name, c -> c.field)
 * -- :282-387.  Writes prod(dims) values of the field's dtype, column-major. */
int vg_rastervalues(vg_sim *s, const char *name, int field, void *out);

/* ---- seeded graph generators of the test models ---------------------------
 * Each plays the part of the model script's add_edge! loop before
 * finish_init! and appends its records, in the loop's call order, to the
 * edge type's staging (no reference counterpart: the reference builds graphs
 * with host loops of add_edge!, src/EdgeMethods.jl:478-522). */
/* agent i (1-based) of type_nr adds k edges i -> t, t uniform in [1, N],
 * t != i; Philox counter (i, j, TAG_EDGE), order (i, j). */
int vg_gen_uniform_out_edges(vg_sim *s, int edge_type, int type_nr, uint32_t k,
                             uint64_t seed);
/* directed Chung-Lu over the agents of type_nr: expected degrees
 * w_i = min(c * i^(-1/(gamma-1)), wmax) with mean `mean`; edge e draws its
 * source and target proportional to w and a weight in (0, 1] into the
 * Float64 field weight_field (-1: none). */
int vg_gen_chung_lu_edges(vg_sim *s, int edge_type, int type_nr, uint64_t nedges,
                          double mean, double gamma, double wmax, uint64_t seed,
                          int weight_field);
/* Staged edge records of an edge type before finish_init!, in call order. */
int vg_read_staged_edges(vg_sim *s, int edge_type, uint64_t *from_out,
                         uint64_t *to_out, void *const *payload_out, uint64_t cap,
                         uint64_t *n_out);

/* ---- self test ----------------------------------------------------------
 * Compares the integer-pipe binary64 add/mul/div used by the gather kernels
 * with the hardware instructions on n generated operand pairs (no reference
 * counterpart).  counts_out[6]: mismatches of add, mul (the general and the
 * gather kernels' form, and scaling by powers of two), div (the general and
 * the gather kernels' form), then the number of out-of-range fallbacks of
 * the general add, mul and div. */
int vg_selftest_fp64(uint64_t n, uint64_t seed, uint64_t *counts_out);

/* Arithmetic throughput on this GPU (no reference counterpart; it measures
 * the pipe the gather kernels' binary64 work runs on).  One launch of
 * `blocks` blocks of 256 threads; in each warp the first active_lanes lanes
 * run iters rounds of 8 independent chains of one operation (mode 0
 * binary64 add, 1 binary64 multiply, 2 binary64 fused multiply-add, 3 the
 * gather kernels' integer-pipe product, 4 a 32-bit integer chain of a
 * multiply-add and an or per round), the
 * other lanes branch around.  *ms_out = the launch's CUDA-event duration,
 * *lane_ops_out = operations performed (lanes x rounds x 8). */
int vg_selftest_rate(int mode, uint32_t blocks, uint32_t iters, uint32_t active_lanes,
                     double *ms_out, double *lane_ops_out);

/* Sorts n generated (key, index) pairs with the library's device radix sort
 * (32-bit keys, or 64-bit keys when wide != 0, key_bits significant bits,
 * bits [const_lo, const_hi) equal in every key) and compares keys and
 * indices with a stable host sort; *mismatch_out = mismatching positions.
 * The sort is what rebuilds every CSR in insertion order (no reference
 * counterpart: Vahana appends to per-agent vectors). */
int vg_selftest_sort(uint64_t n, int key_bits, int wide, int const_lo, int const_hi,
                     uint64_t seed, uint64_t *mismatch_out);

/* Exclusive prefix sum of n generated values (32-bit, or 64-bit when
 * wide != 0; in place when in_place != 0) with the library's single-pass
 * device scan, compared with a host prefix sum; *mismatch_out = mismatching
 * items.  The scan builds row pointers and compaction positions. */
int vg_selftest_scan(uint64_t n, int wide, int in_place, uint64_t seed, uint64_t *mismatch_out);

/* Failure detection without a GPU fault: a look-back scan whose first tile
 * never publishes.  Its successor's bounded wait gives up, records 0x5e02 in
 * the status word and the kernel ends; *status_out = that word, *ms_out =
 * the kernel's duration.  The context stays usable afterwards. */
int vg_selftest_scan_timeout(int *status_out, double *ms_out);

/* Failure detection of the persistent ensemble launch's step waits: two
 * blocks wait for an instance counter that nothing advances, so both
 * bounded waits run out (2^16 polls here); *status_out = the status word (0x5e04), *ms_out =
 * the launch's duration.  The context stays usable. */
int vg_selftest_barrier_timeout(int *status_out, double *ms_out);

/* ---- allocation-free SIR step ---------------------------------------------
 * No counterpart in the reference.  One step of the "sir" transition on
 * device buffers the caller owns, for callers that cannot let a library
 * allocate device memory (a host runtime that owns all device memory and
 * hands in pre-allocated arrays, or code running while another framework
 * captures a CUDA graph).  It calls no cudaMalloc, cudaFree or allocating
 * routine: its only scratch, the table p_k = 1 - (1 - beta)^k, is a fixed
 * file-scope device array of max_in_degree + 1 <= 4096 entries; larger
 * max_in_degree is rejected with VG_ERR_ARG.  Calls share that array, so
 * calls that overlap on the GPU race and must be serialised by the caller.
 * The first call in a CUDA context (the device's primary context, or the
 * context the caller made current) looks the array's address up in that
 * context and caches it under the context's id: make that call before any
 * stream capture.  row_ptr u32[n+1] and src u32 (0-based sources) form the
 * in-edge CSR; state/days are read from the *_in buffers and written to the
 * *_out buffers, which must not overlap the inputs or each other (no
 * in-place step: VG_ERR_ARG); max_in_degree may understate the largest
 * in-degree, in which case the rows beyond the table form the product on
 * the device (same roundings); step is the transition number
 * (num_transitions) that apply! would use; stream is a cudaStream_t. */
int vg_sir_step_noalloc(const uint32_t *row_ptr, const uint32_t *src,
                        const uint8_t *state_in, const int32_t *days_in,
                        uint8_t *state_out, int32_t *days_out, uint64_t n,
                        uint32_t max_in_degree, double beta, int32_t recovery,
                        uint64_t seed, uint32_t step, void *stream);

/* ---- batched ensemble (many independent SIR instances in one arena) ----- */
typedef struct vg_batch vg_batch;
/* Instances i = 0..n-1 with agent counts N[i], out-degree deg[i], infection
 * probability beta[i], recovery steps rec[i], seed seeds[i].  Graphs and
 * initial states are generated on the device from the seeds. */
int vg_batch_create_sir(int n, const int64_t *N, const int32_t *deg,
                        const double *beta, const int32_t *rec,
                        const uint64_t *seeds, int64_t n_init_infected_per_1000,
                        void *stream, vg_batch **out);
/* Advance every instance by `steps` transitions.  mode 0: one launch per
 * step over all instances; mode 1: the same, with the step loop captured
 * once in a CUDA graph and replayed; mode 2: one persistent cooperative
 * launch for all the steps (a block ticket of step t waits until the
 * instances it touches have finished step t - 1; bounded: a
 * wait that runs out is reported as VG_ERR_DEVICE, status 0x5e04); mode 4:
 * one persistent launch of thread-block clusters, each taking packs of
 * whole instances from a counter and stepping a pack through all the steps
 * (the pack's infected-agent masks in the cluster's distributed shared
 * memory, a hardware cluster barrier between steps, no grid-wide barrier);
 * mode 3: mode 1, 2 or 4,
 * whichever the autotuner measured fastest.  The first call runs the
 * autotuner (on copies of the state). */
int vg_batch_step(vg_batch *b, int steps, int mode);
/* The autotuner's choice of form for mode 3 (0 graph replay, 1 persistent
 * grid launch, 2 persistent cluster launch), the persistent grid launch's
 * block size, its degree-bucket threshold (agents with more in-edges take a
 * warp each; 0xFFFFFFFF none), how many agents are above it, and the
 * measured milliseconds per step of the best per-step launch, of the best
 * persistent grid launch and of the best cluster launch (24-step trials on
 * copies of the state; 0 when no cluster shape fits the arena).  Runs the
 * autotuner if it has not run. */
int vg_batch_tuning(vg_batch *b, int *persistent, int *persistent_tpb,
                    uint32_t *bucket_threshold, uint64_t *heavy_agents,
                    double *step_ms_graph, double *step_ms_persistent,
                    double *step_ms_cluster);
/* Overrides the autotuner: mode 3 then takes the graph (persistent = 0),
 * the persistent grid launch (1) or the cluster launch (2), and the
 * persistent grid launch uses this block size (128, 256, 512) and bucket
 * threshold. */
int vg_batch_set_launch(vg_batch *b, int persistent, int persistent_tpb,
                        uint32_t bucket_threshold);
/* Shape of the cluster launch: CTAs per cluster (1, 2, 4, 8), threads per
 * CTA (128, 256, 512) and agents per lane (1, 2); VG_ERR_ARG if a pack's
 * masks would not fit a CTA's shared memory.  The getter also returns the
 * number of clusters launched. */
int vg_batch_set_cluster(vg_batch *b, int ctas, int tpb, int ilp);
int vg_batch_cluster(vg_batch *b, int *ctas, int *tpb, int *ilp,
                     unsigned *clusters);
/* Agents per lane of the per-step launch and of the persistent launch (1, 2
 * or 4: a lane walks the in-edge rows of its agents together).  The setter
 * overrides the autotuner's choice (0 keeps the current value); the getter
 * reads the values in use.  Both run the autotuner if it has not run. */
int vg_batch_set_lanes(vg_batch *b, int per_step, int persistent);
int vg_batch_lanes(vg_batch *b, int *per_step, int *persistent);
/* Plain path for comparison: step instance i alone with the plain kernels. */
int vg_batch_step_one(vg_batch *b, int i, int steps);
int vg_batch_read_states(vg_batch *b, int i, uint8_t *state_out,
                         int32_t *days_out, uint64_t cap, uint64_t *n_out);
/* which = 0: instance i's state in the batched arena; which = 1: the state
 * of instance i's own simulation (advanced by vg_batch_step_one); any other
 * value is VG_ERR_ARG.  n_out (and, for vg_batch_read_graph, both counts)
 * must not be null. */
int vg_batch_read_states2(vg_batch *b, int i, int which, uint8_t *state_out,
                          int32_t *days_out, uint64_t cap, uint64_t *n_out);
int vg_batch_read_graph(vg_batch *b, int i, uint32_t *row_ptr_out,
                        uint32_t *src_out, uint64_t *nrows_out,
                        uint64_t *nedges_out);
/* Totals of the arena and the launch shape the autotuner chose. */
int vg_batch_info(vg_batch *b, uint64_t *agents, uint64_t *edges, int *tpb,
                  int *apt, uint64_t *device_bytes);
int vg_batch_destroy(vg_batch *b);

/* ---- serving loop (no reference counterpart) ------------------------------
 * Simulation jobs of the SIR and the opinion test model arrive over time.
 * A worker thread admits queued jobs, first come first served, while the sum
 * of their estimated device footprints stays within budget_bytes and at most
 * max_active are resident (a job that does not fit an empty server still
 * runs alone).  Each tick advances every resident job by one transition with
 * one launch per model over all of them; a job retires after `steps`
 * transitions.  A job's final state equals the state after `steps` apply!
 * calls on that job built alone (vahana_gb300 models build_sir /
 * build_opinion with the same arguments). */
typedef struct vg_server vg_server;
typedef struct vg_job_spec {
  int model;           /* 0 SIR, 1 bounded-confidence opinion              */
  uint64_t n;          /* agents                                           */
  double mean_degree;  /* SIR: out-degree (rounded); opinion: mean degree  */
  int32_t steps;       /* transitions to run                               */
  uint64_t seed;
  double beta;         /* SIR infection probability                       */
  int32_t recovery;    /* SIR recovery steps                              */
  double eps;          /* opinion confidence bound                        */
  double wmax;         /* opinion: cap of the expected degree (<=0: 1e4)  */
  int keep_state;      /* keep the final state for vg_serve_job_state     */
  int fail_build;      /* failure injection for tests: 1 = the job's build
                        * raises on the host after its simulation and agents
                        * exist; the job is retired with an error status    */
} vg_job_spec;
typedef struct vg_job_result {
  int64_t id;
  int model;
  uint64_t n;
  int32_t steps;
  double arrival_s, admit_s, finish_s; /* seconds since vg_serve_create   */
  uint64_t checksum;                   /* FNV-1a 64 of the final state    */
  double summary;   /* SIR: recovered fraction; opinion: mean opinion      */
  uint64_t device_bytes;
  int status;       /* 0, or the error code of a job whose build failed      */
  char error[124];  /* its message (the server and the other jobs go on)     */
} vg_job_result;
/* The server runs on the device current when it is created. */
int vg_serve_create(uint64_t budget_bytes, int max_active, vg_server **out);
int vg_serve_submit(vg_server *s, const vg_job_spec *spec, int64_t *id_out);
/* Results of jobs finished since the last poll, at most cap. */
int vg_serve_poll(vg_server *s, vg_job_result *out, uint64_t cap, uint64_t *n_out);
/* Final state bytes of a finished job submitted with keep_state (SIR: n
 * state bytes then n Int32 days; opinion: n Float64).  out may be NULL to
 * query the size. */
int vg_serve_job_state(vg_server *s, int64_t id, void *out, uint64_t cap,
                       uint64_t *n_out);
int vg_serve_stats(vg_server *s, uint64_t *queued, uint64_t *active,
                   uint64_t *done, uint64_t *ticks, uint64_t *sim_steps,
                   uint64_t *bytes_in_use);
/* Stop accepting, finish every queued and resident job. */
int vg_serve_drain(vg_server *s);
int vg_serve_destroy(vg_server *s);

#ifdef __cplusplus
}
#endif
#endif /* VAHANA_GB300_H */
