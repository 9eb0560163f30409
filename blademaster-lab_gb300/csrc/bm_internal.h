// Host-side internals shared by the translation units of the library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/blademaster_gb300.h"

struct bm_solver {
    bm_params P;
    bm_buffers B;
    float* viscous_scratch;  // [9][n] inside B.scratch
    int32_t* scan_partials;  // inside B.scratch
    int64_t buckets;
    cudaStream_t side;       // registration and knife integration run here, beside the main chain
    cudaStream_t aux;        // the multi-field node passes run here, beside the single-field ones
    cudaStream_t lists;      // the pair-list build and relists run here, beside the contact pass
    cudaEvent_t fork, join, register_fork, register_join, aux_fork, aux_join, lists_fork, lists_join, labels_fork;
};

struct bm_graph {
    cudaGraph_t graph;
    cudaGraphExec_t exec;
};

namespace bm {

// material
// begin == 0: k_prologue of the same substep already began the registration.
void launch_register(const bm_solver* s, const int64_t* field_codes, int force, cudaStream_t st, int begin = 1);
// aux != nullptr: the multi-field node pass runs on aux beside the single-field
// one (the two write disjoint slots), joined back into st.
void launch_material(const bm_solver* s, int write_sums, cudaStream_t st, cudaStream_t aux = nullptr);
void launch_g2p(const bm_solver* s, cudaStream_t st);
void launch_remap(const bm_solver* s, cudaStream_t st, cudaStream_t aux = nullptr);
// update_F + stress (do_update) and the substep counter (advance_step).
void launch_fupdate(const bm_solver* s, int do_update, int advance_step, cudaStream_t st);
// contact.assign for every knife (nothing when cutting == 0).
void launch_assign(const bm_solver* s, int cut_index, int cutting, cudaStream_t st);
void launch_refresh_stress(const bm_solver* s, cudaStream_t st);
void launch_validate(const bm_solver* s, cudaStream_t st);
void launch_clear_flag(const bm_solver* s, int which, cudaStream_t st);
void launch_plastic_project(float* F, float* Fp, int n, float mu, float yield_stress, int32_t* errors, cudaStream_t st);

// contact
// With registration >= 0 the prologue also begins a topology registration
// (always with 1, when the topology is dirty with 0) for a launch_register
// with begin == 0 later in the substep.
void launch_prologue(const bm_solver* s, int clear_step, cudaStream_t st, int registration = -1);
void launch_rigid(const bm_solver* s, int cut_bits, cudaStream_t st);
void launch_pairs(const bm_solver* s, cudaStream_t st);
// The same launches with the bucket-scan partials (one int per 1024 buckets,
// written before they are read) at `partials`.
void launch_pairs_using(const bm_solver* s, int32_t* partials, cudaStream_t st);
// The three parts of launch_pairs: the full pair-list build (each kernel
// returns at once unless flags[BM_FLAG_PAIR_DIRTY] is set, when `gated`),
// the incremental relist of particles near changed codes (clearing
// flags[BM_FLAG_PAIR_DIRTY] too, when `clear_dirty`), and the pair impulses.
// find_speed: the build finds the largest particle speed itself (inside a
// substep, beside the contact pass) instead of reading buffers.speed.
void launch_pair_build(const bm_solver* s, int32_t* partials, int gated, int find_speed, cudaStream_t st);
// The pair lists of this substep: the full build (gated on a dirty list, or
// always in hash mode) and the relist of changed codes.  With find_speed they
// read positions, velocities, codes and the build state only, none of which
// the contact pass writes, so they may run beside it; the pair impulses
// follow both.
void launch_pair_lists(const bm_solver* s, int32_t* partials, int find_speed, cudaStream_t st);
void launch_relist(const bm_solver* s, int clear_dirty, cudaStream_t st);
void launch_pair_impulses(const bm_solver* s, cudaStream_t st);
void launch_count_embedded(const bm_solver* s, int reset, cudaStream_t st);
// Exclusive prefix sum of `count` ints (one int of `partials` per 1024 of
// them); the total goes to *total_out.  Every kernel returns at once when
// `gate` is non-null and *gate == 0.
void launch_exclusive_scan(const int32_t* in, int32_t* out, int64_t count, int32_t* partials, int32_t* total_out,
                           int32_t* ticket, const int32_t* gate, cudaStream_t st);
// Scratch word 1: the ticket of the scans' last-block pass (zero between scans).
inline int32_t* scan_ticket(const bm_buffers& B) { return B.scratch + 1; }

// held-blade constraint (external tool in hold mode)
void launch_hold(const bm_solver* s, cudaStream_t st);
void launch_blade_query(const float* local, int n, const float* half, float bevel, float* closest, float* normal,
                        float* distance, cudaStream_t st);
void launch_friction(const float* normal, const float* relative, const float* jn, const float* history, int n, float me,
                     float dt, float mus, float mud, float gk, float gc, float* impulse, float* new_history,
                     cudaStream_t st);
void launch_resist_cut(const float* j, const float* x, const float* v, const float* origin, const float* tool_velocity,
                       const float* q, const float* tool_angular, const float* half, float radius, float spacing,
                       float* damage, float threshold, int cutting, uint64_t* work_acc, float* result, int n,
                       cudaStream_t st);
void launch_assign_only(const bm_solver* s, int cut_index, int cutting, cudaStream_t st);

// tool
void launch_tool_step(const bm_solver* s, int mode, int target_index, int advance_step, cudaStream_t st);
void launch_load_external(const bm_solver* s, cudaStream_t st);
void launch_store_interval(const bm_solver* s, cudaStream_t st);
void launch_record_pose(const bm_solver* s, int index, cudaStream_t st);
void launch_tool_mirror(const bm_solver* s, cudaStream_t st);
void launch_read_acc(const bm_solver* s, float* reaction, float* torque, float* board, float* work, cudaStream_t st);
void launch_write_acc(const bm_solver* s, const float* reaction, const float* torque, const float* board,
                      const float* work, cudaStream_t st);
void launch_couple_probe(const int64_t* codes, const float* mass, const float* state, const int32_t* node_start,
                         int nodes, float* result, cudaStream_t st);
void launch_g2p_probe(float* x, float* v, const int32_t* slots, const float* weights, const float* old_v,
                      const float* new_v, int n, float dt, float flip, cudaStream_t st);

// C-ABI error reporting shared by the entry-point translation units: records
// `what` for bm_last_error and returns `code`; check_cuda turns a pending CUDA
// error into BM_ERR_CUDA with `where` in the message.
int fail(int code, const char* what);
int check_cuda(const char* where);

// Tool kernel modes.
enum ToolMode { kToolDrive = 0, kToolFinishExternal = 1, kToolAccumulate = 2, kToolClear = 3 };

}  // namespace bm
