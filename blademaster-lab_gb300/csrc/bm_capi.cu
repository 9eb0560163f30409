// C-ABI of the material substep (include/blademaster_gb300.h): solver
// binding, the per-substep launch sequence of Solver._step_kernels
// (blademaster_warp/solver.py:920-940) and its CUDA-graph capture
// (Solver.prepare, solver.py:975-1019).
#include <stdio.h>
#include <string.h>

#include <initializer_list>
#include <new>
#include <string>
#include <vector>

#include "bm_device.cuh"
#include "bm_internal.h"

namespace {
thread_local std::string g_error;
}  // namespace

namespace bm {

int fail(int code, const char* what) {
    g_error = what;
    return code;
}

int check_cuda(const char* where) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        g_error = std::string(where) + ": " + cudaGetErrorString(e);
        return BM_ERR_CUDA;
    }
    return BM_OK;
}

}  // namespace bm

namespace {

using bm::check_cuda;
using bm::fail;

cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

int64_t tiles_of(const bm_params& P) { return ((int64_t)P.bucket_mask + 1 + 1023) / 1024; }

void layout_scratch(bm_solver* s) {
    // [0] pair reach (float), [1] scan ticket, [8, 25) observation sums and counters (zero between
    // calls), [64 .. 64 + tiles) scan partials, then 9 n floats (viscous stress).
    int32_t* base = s->B.scratch;
    s->scan_partials = base + 64;
    int64_t off = 64 + tiles_of(s->P);
    off = (off + 63) / 64 * 64;
    s->viscous_scratch = reinterpret_cast<float*>(base + off);
}

// Optional CUDA events around each stage of a substep (profiling only).
struct StageTimer {
    cudaEvent_t ev[BM_STAGES + 1];
    bool on = false;
    void mark(int i, cudaStream_t st) {
        if (on) cudaEventRecord(ev[i], st);
    }
};

int64_t kernel_nodes(cudaGraph_t g) {
    size_t n = 0;
    if (cudaGraphGetNodes(g, nullptr, &n) != cudaSuccess) return -1;
    std::vector<cudaGraphNode_t> nodes(n);
    if (n && cudaGraphGetNodes(g, nodes.data(), &n) != cudaSuccess) return -1;
    int64_t kernels = 0;
    for (size_t i = 0; i < n; ++i) {
        cudaGraphNodeType type;
        if (cudaGraphNodeGetType(nodes[i], &type) != cudaSuccess) return -1;
        if (type == cudaGraphNodeTypeKernel) ++kernels;
    }
    return kernels;
}

// One batch of substeps on stream st.
int run_batch(bm_solver* s, const bm_step_args* a, cudaStream_t st, StageTimer* timer = nullptr,
              float* stage_ms = nullptr) {
    const bm_params& P = s->P;
    const int64_t* field_codes = a->single_field ? s->B.zero_codes : s->B.codes;
    const bool force_topology = !P.cache_topology;
    StageTimer none;
    StageTimer& t = timer ? *timer : none;
    if (a->external_load) bm::launch_load_external(s, st);
    if (a->record_samples) bm::launch_record_pose(s, 0, st);
    for (int i = 0; i < a->steps; ++i) {
        t.mark(0, st);
        bm::launch_prologue(s, P.external_tool ? 0 : 1, st, force_topology ? 1 : 0);
        // The topology registration reads only the codes of the last substep and
        // writes only the field tables, which the contact and pair passes do not
        // touch: outside profiling it runs on the side stream beside them.
        const bool overlap = !t.on;
        if (overlap) {
            cudaEventRecord(s->register_fork, st);
            cudaStreamWaitEvent(s->side, s->register_fork, 0);
            bm::launch_register(s, field_codes, force_topology ? 1 : 0, s->side, 0);
            cudaEventRecord(s->register_join, s->side);
        }
        // The pair lists (full build when dirty, relists of changed codes) read
        // positions, velocities and codes, which the contact pass does not
        // write: outside profiling they run on their own stream beside it.
        if (overlap) {
            cudaEventRecord(s->lists_fork, st);
            cudaStreamWaitEvent(s->lists, s->lists_fork, 0);
            bm::launch_pair_lists(s, s->scan_partials, 1, s->lists);
            cudaEventRecord(s->lists_join, s->lists);
        }
        t.mark(1, st);
        bm::launch_rigid(s, a->cut_bits, st);
        t.mark(2, st);
        // The knife integration needs only this substep's reactions and is read
        // only by the side labels and the next substep, so (outside
        // external mode, where the grid constraint may still change the
        // reaction) it runs on a side stream concurrently with the transfers.
        int mode = bm::kToolDrive;
        if (P.external_tool) mode = bm::kToolFinishExternal;
        else if (P.accumulate_tool_impulses) mode = bm::kToolAccumulate;
        const bool fork = !t.on && !P.external_tool;
        if (fork) {
            cudaEventRecord(s->fork, st);
            cudaStreamWaitEvent(s->side, s->fork, 0);
            bm::launch_tool_step(s, mode, a->use_targets ? i : 0, 1, s->side);
            cudaEventRecord(s->join, s->side);
        }
        if (overlap) cudaStreamWaitEvent(st, s->lists_join, 0);
        else bm::launch_pair_lists(s, s->scan_partials, 1, st);
        bm::launch_pair_impulses(s, st);
        t.mark(3, st);
        if (overlap) cudaStreamWaitEvent(st, s->register_join, 0);
        else bm::launch_register(s, field_codes, force_topology ? 1 : 0, st, 0);
        t.mark(4, st);
        bm::launch_material(s, 0, st, overlap ? s->aux : nullptr);
        if (P.external_tool && !P.predict) bm::launch_hold(s, st);
        t.mark(5, st);
        bm::launch_g2p(s, st);
        // The side labels read the knife after its step and x, v after G2P; they
        // write only codes and the next substep's relist and registration work
        // lists, which neither the remap nor the F update reads.  Outside
        // profiling they run on the side stream after the knife, beside those
        // passes, and the next substep starts after both.
        if (fork) {
            cudaEventRecord(s->labels_fork, st);
            cudaStreamWaitEvent(s->side, s->labels_fork, 0);
            bm::launch_assign(s, a->cut_index, a->cut_bits != 0, s->side);
            cudaEventRecord(s->join, s->side);
        }
        t.mark(6, st);
        bm::launch_remap(s, st, overlap ? s->aux : nullptr);
        t.mark(7, st);
        if (!fork) bm::launch_tool_step(s, mode, a->use_targets ? i : 0, 1, st);
        t.mark(8, st);
        bm::launch_fupdate(s, 1, 1, st);
        t.mark(9, st);
        if (fork) cudaStreamWaitEvent(st, s->join, 0);
        else bm::launch_assign(s, a->cut_index, a->cut_bits != 0, st);
        t.mark(10, st);
        if (t.on) {
            if (cudaEventSynchronize(t.ev[BM_STAGES]) != cudaSuccess) return check_cuda("profiled substep");
            for (int k = 0; k < BM_STAGES; ++k) {
                float ms = 0.0f;
                cudaEventElapsedTime(&ms, t.ev[k], t.ev[k + 1]);
                stage_ms[k] += ms;
            }
        }
        if (a->record_samples && (!a->hold_pose || i == a->steps - 1))
            bm::launch_record_pose(s, a->hold_pose ? 1 : i + 1, st);
    }
    if (a->external_finish) {
        bm::launch_validate(s, st);
        bm::launch_store_interval(s, st);
    }
    return check_cuda("substeps");
}

}  // namespace


extern "C" {

uint32_t bm_params_size(void) { return (uint32_t)sizeof(bm_params); }
uint32_t bm_buffers_size(void) { return (uint32_t)sizeof(bm_buffers); }
uint32_t bm_step_args_size(void) { return (uint32_t)sizeof(bm_step_args); }
const char* bm_last_error(void) { return g_error.c_str(); }
const char* bm_version(void) { return "blademaster_gb300 0.1 sm_103a"; }

int64_t bm_scratch_words(const bm_params* P) {
    if (!P) return -1;
    int64_t off = 64 + tiles_of(*P);
    off = (off + 63) / 64 * 64;
    return off + 9 * (int64_t)P->n + 64;
}

int bm_solver_create(const bm_params* params, const bm_buffers* buffers, bm_solver** out) {
    if (!params || !buffers || !out) return fail(BM_ERR_ARGUMENT, "null argument");
    const bm_params& P = *params;
    if (P.n < 1 || P.node_count < 1 || P.active_nodes < 1 || P.fmax < 1 || P.fmax > 255)
        return fail(BM_ERR_ARGUMENT, "invalid sizes (n, node_count, active_nodes, fmax in [1, 255])");
    if (P.tool_count < 1 || P.tool_count > BM_MAX_TOOLS) return fail(BM_ERR_ARGUMENT, "tool_count must be in [1, 16]");
    if ((P.bucket_mask & (P.bucket_mask + 1)) != 0 || P.bucket_mask < 1) return fail(BM_ERR_ARGUMENT, "bucket_mask must be 2^k - 1");
    if (P.pair_capacity < 16) return fail(BM_ERR_ARGUMENT, "pair_capacity too small");
    if ((int64_t)P.node_dims[0] * P.node_dims[1] * P.node_dims[2] != P.node_count)
        return fail(BM_ERR_ARGUMENT, "node_dims do not match node_count");
    const void* required[] = {buffers->x, buffers->v, buffers->ref, buffers->F, buffers->Fp, buffers->stress,
                              buffers->codes, buffers->zero_codes, buffers->damage, buffers->histories,
                              buffers->impulses, buffers->stencil_id, buffers->stencil_w, buffers->stencil_g,
                              buffers->base_node, buffers->fidx, buffers->cell_start, buffers->active,
                              buffers->nfield, buffers->fcode, buffers->fones, buffers->ftwos, buffers->grid_mass,
                              buffers->momentum, buffers->grid_impulse, buffers->old_v, buffers->new_v,
                              buffers->remapped, buffers->remap_v, buffers->built_x, buffers->built_codes,
                              buffers->partners, buffers->partner_count, buffers->candidates, buffers->bucket_start,
                              buffers->bucket_items, buffers->bucket_fill, buffers->particle_bucket,
                              buffers->pair_keys, buffers->pair_history, buffers->pair_used, buffers->pair_count,
                              buffers->tool, buffers->tool_f, buffers->mobility, buffers->acc, buffers->interval,
                              buffers->table_impulse, buffers->speed, buffers->errors, buffers->flags,
                              buffers->targets, buffers->rotations, buffers->packed, buffers->result,
                              buffers->scratch, buffers->cell_part, buffers->cell_field, buffers->hist_mask,
                              buffers->changed, buffers->relist, buffers->relist_list, buffers->listed,
                              buffers->multi_nodes, buffers->mixed_cells,
                              buffers->particle_key, buffers->bucket_key, buffers->bucket_pos,
                              buffers->reg_node_mark, buffers->reg_nodes, buffers->reg_cell_mark, buffers->reg_cells};
    for (const void* ptr : required)
        if (!ptr) return fail(BM_ERR_ARGUMENT, "a required buffer is null");
    if (P.maxwell && !buffers->viscous) return fail(BM_ERR_ARGUMENT, "maxwell requires the viscous buffer");
    if (P.external_tool && !P.predict) {
        const void* hold[] = {buffers->hold, buffers->hold_mark, buffers->hold_pos, buffers->hold_list,
                              buffers->hold_entry, buffers->hold_node_start, buffers->hold_nodes, buffers->hold_node_mark};
        for (const void* ptr : hold)
            if (!ptr) return fail(BM_ERR_ARGUMENT, "hold mode requires the hold_* buffers");
    }
    bm_solver* s = new (std::nothrow) bm_solver;
    if (!s) return fail(BM_ERR_STATE, "out of host memory");
    s->P = P;
    s->B = *buffers;
    s->buckets = (int64_t)P.bucket_mask + 1;
    layout_scratch(s);
    s->side = s->aux = s->lists = nullptr;
    s->fork = s->join = s->register_fork = s->register_join = s->aux_fork = s->aux_join = nullptr;
    s->lists_fork = s->lists_join = s->labels_fork = nullptr;
    if (cudaMemset(s->B.scratch + 1, 0, 63 * sizeof(int32_t)) != cudaSuccess ||
        cudaStreamCreateWithFlags(&s->side, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&s->aux, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&s->lists, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&s->lists_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&s->lists_join, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&s->labels_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&s->aux_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&s->aux_join, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&s->fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&s->join, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&s->register_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&s->register_join, cudaEventDisableTiming) != cudaSuccess) {
        const int rc = check_cuda("solver streams");
        for (cudaStream_t q : {s->side, s->aux, s->lists})
            if (q) cudaStreamDestroy(q);
        for (cudaEvent_t e : {s->fork, s->join, s->register_fork, s->register_join, s->aux_fork, s->aux_join,
                              s->lists_fork, s->lists_join, s->labels_fork})
            if (e) cudaEventDestroy(e);
        delete s;
        return rc;
    }
    *out = s;
    return BM_OK;
}

int bm_solver_destroy(bm_solver* s) {
    if (!s) return BM_OK;
    for (cudaStream_t q : {s->side, s->aux, s->lists}) {
        cudaStreamSynchronize(q);
        cudaStreamDestroy(q);
    }
    for (cudaEvent_t e : {s->fork, s->join, s->register_fork, s->register_join, s->aux_fork, s->aux_join,
                          s->lists_fork, s->lists_join, s->labels_fork})
        cudaEventDestroy(e);
    delete s;
    return BM_OK;
}

int bm_refresh_stress(bm_solver* s, void* stream) {
    if (!s) return fail(BM_ERR_ARGUMENT, "null solver");
    bm::launch_refresh_stress(s, as_stream(stream));
    return check_cuda("refresh_stress");
}

int bm_register_topology(bm_solver* s, int single_field, void* stream) {
    if (!s) return fail(BM_ERR_ARGUMENT, "null solver");
    cudaStream_t st = as_stream(stream);
    bm::launch_register(s, single_field ? s->B.zero_codes : s->B.codes, 1, st);
    bm::launch_clear_flag(s, BM_FLAG_TOPOLOGY_DIRTY, st);
    return check_cuda("register_topology");
}

int bm_material_step(bm_solver* s, int single_field, void* stream) {
    if (!s) return fail(BM_ERR_ARGUMENT, "null solver");
    cudaStream_t st = as_stream(stream);
    bm::launch_register(s, single_field ? s->B.zero_codes : s->B.codes, s->P.cache_topology ? 0 : 1, st);
    bm::launch_material(s, 1, st);
    if (s->P.external_tool && !s->P.predict) bm::launch_hold(s, st);
    bm::launch_g2p(s, st);
    bm::launch_remap(s, st);
    bm::launch_fupdate(s, 1, 0, st);
    return check_cuda("material_step");
}

int bm_hold_constraint(bm_solver* s, void* stream) {
    if (!s) return fail(BM_ERR_ARGUMENT, "null solver");
    if (!s->P.external_tool || s->P.predict) return fail(BM_ERR_STATE, "the held-blade constraint needs an external tool in hold mode");
    bm::launch_hold(s, as_stream(stream));
    return check_cuda("hold_constraint");
}

int bm_rigid_contacts(bm_solver* s, int cut_bits, void* stream) {
    if (!s) return fail(BM_ERR_ARGUMENT, "null solver");
    bm::launch_rigid(s, cut_bits, as_stream(stream));
    return check_cuda("rigid_contacts");
}

int bm_particle_contacts(bm_solver* s, void* stream) {
    if (!s) return fail(BM_ERR_ARGUMENT, "null solver");
    cudaStream_t st = as_stream(stream);
    bm::launch_prologue(s, 0, st);
    bm::launch_pairs(s, st);
    return check_cuda("particle_contacts");
}

int bm_assign_sides(bm_solver* s, int cut_index, int cutting, void* stream) {
    if (!s) return fail(BM_ERR_ARGUMENT, "null solver");
    bm::launch_assign(s, cut_index, cutting, as_stream(stream));
    return check_cuda("assign_sides");
}

int bm_drive_tool(bm_solver* s, int index, void* stream) {
    if (!s) return fail(BM_ERR_ARGUMENT, "null solver");
    bm::launch_tool_step(s, bm::kToolDrive, index, 0, as_stream(stream));
    return check_cuda("drive_tool");
}

int bm_finish_external(bm_solver* s, void* stream) {
    if (!s) return fail(BM_ERR_ARGUMENT, "null solver");
    bm::launch_tool_step(s, bm::kToolFinishExternal, 0, 0, as_stream(stream));
    return check_cuda("finish_external");
}

int bm_accumulate_tool_impulses(bm_solver* s, void* stream) {
    if (!s) return fail(BM_ERR_ARGUMENT, "null solver");
    bm::launch_tool_step(s, bm::kToolAccumulate, 0, 0, as_stream(stream));
    return check_cuda("accumulate_tool_impulses");
}

int bm_clear_step(bm_solver* s, void* stream) {
    if (!s) return fail(BM_ERR_ARGUMENT, "null solver");
    bm::launch_tool_step(s, bm::kToolClear, 0, 0, as_stream(stream));
    return check_cuda("clear_step");
}

int bm_substeps(bm_solver* s, const bm_step_args* args, void* stream) {
    if (!s || !args) return fail(BM_ERR_ARGUMENT, "null argument");
    if (args->steps < 0) return fail(BM_ERR_ARGUMENT, "steps must be non-negative");
    return run_batch(s, args, as_stream(stream));
}

int bm_substeps_profiled(bm_solver* s, const bm_step_args* args, float* stage_ms, void* stream) {
    if (!s || !args || !stage_ms) return fail(BM_ERR_ARGUMENT, "null argument");
    StageTimer timer;
    for (int k = 0; k <= BM_STAGES; ++k) cudaEventCreate(&timer.ev[k]);
    for (int k = 0; k < BM_STAGES; ++k) stage_ms[k] = 0.0f;
    timer.on = true;
    int rc = run_batch(s, args, as_stream(stream), &timer, stage_ms);
    for (int k = 0; k <= BM_STAGES; ++k) cudaEventDestroy(timer.ev[k]);
    return rc;
}

int bm_graph_create(bm_solver* s, const bm_step_args* args, void* stream, bm_graph** out) {
    if (!s || !args || !out) return fail(BM_ERR_ARGUMENT, "null argument");
    (void)stream;
    cudaStream_t cap;
    if (cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking) != cudaSuccess) return check_cuda("stream create");
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
        cudaStreamDestroy(cap);
        return check_cuda("begin capture");
    }
    int rc = run_batch(s, args, cap);
    e = cudaStreamEndCapture(cap, &graph);
    cudaStreamDestroy(cap);
    if (rc != BM_OK) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
    }
    if (e != cudaSuccess) return check_cuda("end capture");
    cudaGraphExec_t exec;
    if (cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) {
        cudaGraphDestroy(graph);
        return check_cuda("graph instantiate");
    }
    bm_graph* g = new (std::nothrow) bm_graph;
    if (!g) {
        cudaGraphExecDestroy(exec);
        cudaGraphDestroy(graph);
        return fail(BM_ERR_STATE, "out of host memory");
    }
    g->graph = graph;
    g->exec = exec;
    *out = g;
    return BM_OK;
}

int bm_batch_graph_create(bm_solver* const* solvers, const bm_step_args* args, int count, int lanes, void* stream,
                          bm_graph** out) {
    if (!solvers || !args || !out || count < 1 || lanes < 1) return fail(BM_ERR_ARGUMENT, "invalid arguments");
    for (int i = 0; i < count; ++i)
        if (!solvers[i] || args[i].steps < 0) return fail(BM_ERR_ARGUMENT, "null solver or negative steps");
    (void)stream;
    if (lanes > count) lanes = count;
    std::vector<cudaStream_t> lane(lanes, nullptr);
    std::vector<cudaEvent_t> done(lanes, nullptr);
    cudaStream_t origin = nullptr;
    cudaEvent_t start = nullptr;
    auto release = [&]() {
        for (int l = 0; l < lanes; ++l) {
            if (lane[l]) cudaStreamDestroy(lane[l]);
            if (done[l]) cudaEventDestroy(done[l]);
        }
        if (origin) cudaStreamDestroy(origin);
        if (start) cudaEventDestroy(start);
    };
    bool ok = cudaStreamCreateWithFlags(&origin, cudaStreamNonBlocking) == cudaSuccess &&
              cudaEventCreateWithFlags(&start, cudaEventDisableTiming) == cudaSuccess;
    for (int l = 0; ok && l < lanes; ++l)
        ok = cudaStreamCreateWithFlags(&lane[l], cudaStreamNonBlocking) == cudaSuccess &&
             cudaEventCreateWithFlags(&done[l], cudaEventDisableTiming) == cudaSuccess;
    if (!ok) {
        release();
        return check_cuda("batch streams");
    }
    cudaGraph_t graph = nullptr;
    if (cudaStreamBeginCapture(origin, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        release();
        return check_cuda("begin capture");
    }
    cudaEventRecord(start, origin);
    for (int l = 0; l < lanes; ++l) cudaStreamWaitEvent(lane[l], start, 0);
    int rc = BM_OK;
    for (int i = 0; i < count && rc == BM_OK; ++i)
        rc = run_batch(solvers[i], &args[i], lane[i % lanes]);
    for (int l = 0; l < lanes; ++l) {
        cudaEventRecord(done[l], lane[l]);
        cudaStreamWaitEvent(origin, done[l], 0);
    }
    const cudaError_t e = cudaStreamEndCapture(origin, &graph);
    release();
    if (rc != BM_OK) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
    }
    if (e != cudaSuccess) return check_cuda("end capture");
    cudaGraphExec_t exec;
    if (cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) {
        cudaGraphDestroy(graph);
        return check_cuda("graph instantiate");
    }
    bm_graph* g = new (std::nothrow) bm_graph;
    if (!g) {
        cudaGraphExecDestroy(exec);
        cudaGraphDestroy(graph);
        return fail(BM_ERR_STATE, "out of host memory");
    }
    g->graph = graph;
    g->exec = exec;
    *out = g;
    return BM_OK;
}

int bm_graph_launch(bm_graph* g, void* stream) {
    if (!g) return fail(BM_ERR_ARGUMENT, "null graph");
    cudaGraphLaunch(g->exec, as_stream(stream));
    return check_cuda("graph launch");
}

int bm_graph_destroy(bm_graph* g) {
    if (!g) return BM_OK;
    cudaGraphExecDestroy(g->exec);
    cudaGraphDestroy(g->graph);
    delete g;
    return BM_OK;
}

int bm_graph_kernel_count(const bm_graph* g, int64_t* count) {
    if (!g || !count) return fail(BM_ERR_ARGUMENT, "null argument");
    const int64_t kernels = kernel_nodes(g->graph);
    if (kernels < 0) return check_cuda("graph nodes");
    *count = kernels;
    return BM_OK;
}

int bm_count_embedded(bm_solver* s, int reset, void* stream) {
    if (!s) return fail(BM_ERR_ARGUMENT, "null solver");
    bm::launch_count_embedded(s, reset, as_stream(stream));
    return check_cuda("count_embedded");
}

int bm_validate_interval(bm_solver* s, void* stream) {
    if (!s) return fail(BM_ERR_ARGUMENT, "null solver");
    bm::launch_validate(s, as_stream(stream));
    return check_cuda("validate_interval");
}

int bm_read_accumulators(bm_solver* s, float* reaction, float* torque, float* board, float* work, void* stream) {
    if (!s) return fail(BM_ERR_ARGUMENT, "null solver");
    bm::launch_read_acc(s, reaction, torque, board, work, as_stream(stream));
    return check_cuda("read_accumulators");
}

int bm_write_accumulators(bm_solver* s, const float* reaction, const float* torque, const float* board,
                          const float* work, void* stream) {
    if (!s) return fail(BM_ERR_ARGUMENT, "null solver");
    bm::launch_write_acc(s, reaction, torque, board, work, as_stream(stream));
    return check_cuda("write_accumulators");
}

int bm_sync_tool_mirror(bm_solver* s, void* stream) {
    if (!s) return fail(BM_ERR_ARGUMENT, "null solver");
    bm::launch_tool_mirror(s, as_stream(stream));
    return check_cuda("sync_tool_mirror");
}

int bm_blade_query(const float* local, int n, const float* half, float bevel, float* closest, float* normal,
                   float* distance, void* stream) {
    if (n < 0 || !half) return fail(BM_ERR_ARGUMENT, "invalid arguments");
    if (n == 0) return BM_OK;
    bm::launch_blade_query(local, n, half, bevel, closest, normal, distance, as_stream(stream));
    return check_cuda("blade_query");
}

int bm_friction(const float* normal, const float* relative, const float* jn, const float* history, int n, float me,
                float dt, float mus, float mud, float gk, float gc, float* impulse, float* new_history, void* stream) {
    if (n < 0) return fail(BM_ERR_ARGUMENT, "invalid arguments");
    if (n == 0) return BM_OK;
    bm::launch_friction(normal, relative, jn, history, n, me, dt, mus, mud, gk, gc, impulse, new_history,
                        as_stream(stream));
    return check_cuda("friction");
}

int bm_couple_fields(const int64_t* codes, const float* mass, const float* state, const int32_t* node_start, int nodes,
                     float* result, void* stream) {
    if (nodes < 0) return fail(BM_ERR_ARGUMENT, "invalid arguments");
    if (nodes == 0) return BM_OK;
    bm::launch_couple_probe(codes, mass, state, node_start, nodes, result, as_stream(stream));
    return check_cuda("couple_fields");
}

int bm_g2p_probe(float* x, float* v, const int32_t* slots, const float* weights, const float* old_v,
                 const float* new_v, int n, float dt, float flip, void* stream) {
    if (n < 0) return fail(BM_ERR_ARGUMENT, "invalid arguments");
    if (n == 0) return BM_OK;
    bm::launch_g2p_probe(x, v, slots, weights, old_v, new_v, n, dt, flip, as_stream(stream));
    return check_cuda("g2p_probe");
}

int bm_resist_cut_probe(const float* j, const float* x, const float* v, const float* origin,
                        const float* tool_velocity, const float* q, const float* tool_angular, const float* half,
                        float radius, float spacing, float* damage, float threshold, int cutting, uint64_t* work_acc,
                        float* result, int n, void* stream) {
    if (n < 0 || !half) return fail(BM_ERR_ARGUMENT, "invalid arguments");
    if (n == 0) return BM_OK;
    bm::launch_resist_cut(j, x, v, origin, tool_velocity, q, tool_angular, half, radius, spacing, damage, threshold,
                          cutting, work_acc, result, n, as_stream(stream));
    return check_cuda("resist_cut");
}

int bm_plastic_project(float* F, float* Fp, int n, float mu, float yield_stress, int32_t* errors, void* stream) {
    if (n < 0) return fail(BM_ERR_ARGUMENT, "invalid arguments");
    if (n == 0) return BM_OK;
    bm::launch_plastic_project(F, Fp, n, mu, yield_stress, errors, as_stream(stream));
    return check_cuda("plastic_project");
}

}  // extern "C"
