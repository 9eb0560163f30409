/*
 * blademaster_gb300 C-ABI: the material substep of BladeMaster-Lab's TLMPM
 * cutting solver on one GB300 (sm_103a).
 *
 * The reference (Ju6276/BladeMaster-Lab, Python + NVIDIA Warp) has no C
 * interface: its hot path is a fixed sequence of Warp kernel launches driven
 * by blademaster_warp/solver.py.  Each entry point below replaces one of those
 * launches (or one Solver method that launches several), named after it, and
 * is what a host binding (ctypes here, or cgo / JNI / N-API) calls.
 *
 * Ownership: every device buffer is allocated by the caller (PyTorch on the
 * Python side) and passed once in bm_buffers; addresses must stay valid and
 * fixed for the solver's lifetime, because captured CUDA graphs embed them
 * (the reference relies on the same rule, solver.py:986-990).  No entry point
 * allocates device memory except bm_graph_create (graph objects).
 *
 * Errors: every function returns 0 on success or a BM_ERR_* class; the
 * message of the last failure on the calling thread is bm_last_error().
 * Device-detected errors are counted in buffers.errors[3] = [storage
 * overflow, inverted material, coincident proxies], the reference's counters
 * (solver.py:307, raised at solver.py:1022-1026).
 *
 * Threading: a solver is driven from one host thread on one stream at a time
 * (solver.py:158-162 has the same contract).
 */
#ifndef BLADEMASTER_GB300_H
#define BLADEMASTER_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BM_OK 0
#define BM_ERR_ARGUMENT 1
#define BM_ERR_CUDA 2
#define BM_ERR_STATE 3

/* Bits of the `cutting` argument (contact.py:15-18). */
#define BM_CUT_ON 1
#define BM_CUT_ADVANCE 2
#define BM_CUT_HOLD 4

#define BM_MAX_TOOLS 16
/* Float32 knife record: pos 3, vel 3, rot 4, omega 3, |vel| 1, |omega| * blade radius 1,
 * edge centre 3, cutting direction 3, edge velocity 3, knife axes 9, padding 3. */
#define BM_TOOL_F_WORDS 36
#define BM_PAIR_LANES 64

/* Scalars of one solver: Config (solver.py:12-149) plus the derived
 * constants of Solver.__init__ (solver.py:164-200).  float fields are the
 * float32 values the particle kernels use; *_d fields are float64 copies used
 * by the single-thread tool integration. */
typedef struct bm_params {
    int32_t n;                 /* particles */
    int32_t node_count;        /* nodes of the reference grid, prod(cells + 1) */
    int32_t node_dims[3];
    int32_t cell_dims[3];
    int32_t active_nodes;      /* nodes touched by at least one particle */
    int32_t fmax;              /* field slots per node (slot = f * node_count + node) */
    int32_t stencil_rows;      /* rows of the stencil table */
    int32_t tool_count;
    int32_t pair_capacity;     /* friction-history hash table size (power of two) */
    int32_t bucket_mask;       /* pair search buckets - 1 (power of two) */
    int32_t candidate_capacity;
    int32_t pad_sizes;
    /* mode flags */
    int32_t tool_model;        /* -1 external, 0 guided, 1 free/servo (solver.py:571-576) */
    int32_t external_tool;
    int32_t predict;           /* tool_substep == predict */
    int32_t free_blade;
    int32_t lock_rotation;     /* guided knife: not free and not pose servo */
    int32_t accumulate_tool_impulses;
    int32_t plastic;           /* yield_stress > 0 */
    int32_t use_fp;            /* Fp may differ from identity */
    int32_t maxwell;
    int32_t viscous;           /* dynamic_viscosity > 0 */
    int32_t pair_search;       /* 0 skin list rebuilt on demand, 1 rebuilt every substep */
    int32_t cache_topology;    /* register fields only when a cut code changed */
    /* material */
    float dt, spacing, mass, volume, radius, mu, lam, mu_maxwell, maxwell_relax;
    float yield_stress, flip, dynamic_viscosity;
    /* contact */
    float normal_scale, tangent_stiffness, friction_static, friction_dynamic, tangent_damping;
    float board_scale, board_half[2];
    float half[3], bevel, blade_offset, blade_mass, inertia_inv[3], threshold;
    float pair_skin, pad1;
    /* tool drive, float64 */
    double dt_d, blade_mass_d, half_d[3], bevel_d, inertia_inv_d[3];
    double drive_stiffness, drive_damping, drive_force_limit, rot_stiffness, rot_damping, friction_dynamic_d;
    double board_half_d[2];
} bm_params;

/* Device buffers (caller-owned).  Particle arrays are in device order
 * (sorted by reference cell) and structure-of-arrays: a "[3][n]" array holds
 * all x components, then all y, then all z. */
typedef struct bm_buffers {
    /* particles */
    float* x;            /* [3][n] */
    float* v;            /* [3][n] */
    float* ref;          /* [3][n] reference positions */
    float* F;            /* [9][n] row-major components */
    float* Fp;           /* [9][n] */
    float* stress;       /* [9][n] first Piola stress of the current F, Fp */
    double* viscous;     /* [9][n] Fv - I of the Maxwell branch */
    int64_t* codes;      /* [n] ternary cut codes */
    int64_t* zero_codes; /* [n] all zero: transfers of the single-field baseline */
    float* damage;       /* [tools][n] */
    float* histories;    /* [1 + tools][3][n]: row 0 board, row 1 + k knife k */
    float* impulses;     /* [3][n] contact impulses of this substep */
    int32_t* stencil_id; /* [n] row of the stencil table */
    float* stencil_w;    /* [rows][8] */
    float* stencil_g;    /* [rows][8][3] */
    int32_t* base_node;  /* [n] node of the particle's cell corner (0, 0, 0) */
    uint64_t* fidx;      /* [n] 8 x 8-bit field index of each stencil node */
    /* grid */
    int32_t* cell_start; /* [cells + 1] particles of cell c are [cell_start[c], cell_start[c+1]) */
    int32_t* active;     /* [active_nodes] node ids */
    int32_t* nfield;     /* [node_count] fields registered at each node */
    int64_t* fcode;      /* [fmax][node_count] code of each field (ascending per node) */
    uint64_t* fones;     /* [fmax][node_count] digit masks of the code */
    uint64_t* ftwos;     /* [fmax][node_count] */
    float* grid_mass;    /* [fmax * node_count] */
    float* momentum;     /* [3][fmax * node_count] */
    float* grid_impulse; /* [3][fmax * node_count] */
    float* old_v;        /* [3][fmax * node_count] */
    float* new_v;        /* [3][fmax * node_count] */
    float* remapped;     /* [3][fmax * node_count] remapped momentum (multi-field nodes) */
    float* remap_v;      /* [3][fmax * node_count] coupled remapped momentum / mass */
    float* cell_part;    /* [7][8][node_count] cell-corner partial sums: from the cell whose corner a is node n */
    uint8_t* cell_field; /* [node_count][8] field index of a uniform cell corner, 255 mixed, 254 no cell */
    int32_t* multi_nodes;/* [active_nodes] nodes with more than one field */
    int32_t* mixed_cells;/* [cells] cells whose particles map to different fields at some corner */
    /* pair contact */
    float* built_x;      /* [3][n] */
    int64_t* built_codes;/* [n] */
    int32_t* partners;   /* [n][BM_PAIR_LANES] */
    int32_t* partner_count; /* [n]; -1 overflow */
    int32_t* candidates; /* [candidate_capacity] particles with partners */
    int32_t* bucket_start;  /* [buckets + 1] */
    int32_t* bucket_items;  /* [n] */
    int32_t* bucket_fill;   /* [buckets] */
    int32_t* particle_bucket; /* [n] */
    int64_t* particle_key;  /* [n] packed cell of the particle at the last build */
    int64_t* bucket_key;    /* [n] packed cell of each bucket item */
    float* bucket_pos;      /* [n][4] position of each bucket item at the last build */
    int64_t* pair_keys;  /* [2][pair_capacity] */
    float* pair_history; /* [2][pair_capacity][3] */
    int32_t* pair_used;  /* [2][pair_capacity] */
    int32_t* pair_count; /* [2] */
    int32_t* changed;    /* [n] particles whose cut code changed since the last list update */
    int32_t* relist;     /* [n] 1 while a particle's partner list awaits recomputation */
    int32_t* relist_list;/* [n] those particles */
    int32_t* listed;     /* [n] 1 if the particle is in candidates */
    /* incremental topology registration (codes changed by side labelling only) */
    int32_t* reg_node_mark; /* [node_count] 1 while a node awaits registration; zero between substeps */
    int32_t* reg_nodes;     /* [node_count] those nodes */
    int32_t* reg_cell_mark; /* [cells] 1 while a cell's particles await new field indices; zero between substeps */
    int32_t* reg_cells;     /* [cells] those cells */
    /* tool and scalar state */
    double* tool;        /* [tools][13]: pos 3, vel 3, rot xyzw 4, omega 3 */
    float* tool_f;       /* [tools][BM_TOOL_F_WORDS] float32 mirror read by particle kernels */
    uint16_t* hist_mask; /* [n] bit 0: board history may be non-zero; bit 1 + k: knife k's */
    float* mobility;     /* [36] */
    uint64_t* acc;       /* 128-bit accumulators, see BM_ACC_* */
    double* interval;    /* [6] interval impulse 3, angular impulse about the world origin 3 */
    double* table_impulse; /* [tools][3] */
    float* speed;        /* [1] max particle speed this substep */
    int32_t* errors;     /* [3] */
    int32_t* flags;      /* see BM_FLAG_* */
    float* targets;      /* [steps][3] per-substep edge targets (driven knives) */
    float* rotations;    /* [steps][4] per-substep target orientations */
    float* packed;       /* [49] external tool state */
    float* result;       /* [10 + 7 * samples] interval result */
    int32_t* scratch;    /* [scratch_len] scan workspace */
    /* held-blade grid constraint (external tool with tool_substep "hold" only; may be null otherwise) */
    float* hold;         /* [11][n]: entry side, normal xyz, lever xyz, rhs, row bound, impulse, extrapolated */
    int32_t* hold_mark;  /* [n] 1 if the particle is a constraint contact this substep */
    int32_t* hold_pos;   /* [n] exclusive prefix sum of hold_mark */
    int32_t* hold_list;  /* [n] contacts in ascending particle order */
    int32_t* hold_entry; /* [8 n] contacts at each listed node, particle << 3 | corner, ascending particle */
    int32_t* hold_node_start; /* [node_count + 1] */
    int32_t* hold_nodes; /* [node_count] grid nodes the contacts touch */
    int32_t* hold_node_mark; /* [node_count] all zero between substeps */
} bm_buffers;

/* Layout of buffers.acc: pairs of uint64 (lo, hi), 2^-96 fixed point. */
#define BM_ACC_REACTION(k) (2 * (3 * (k)))          /* knife k: 3 components */
#define BM_ACC_TORQUE(k) (2 * (3 * BM_MAX_TOOLS + 3 * (k)))
#define BM_ACC_BOARD (2 * (6 * BM_MAX_TOOLS))
#define BM_ACC_WORK (2 * (6 * BM_MAX_TOOLS + 3))
#define BM_ACC_WORDS (2 * (6 * BM_MAX_TOOLS + 4))

/* Layout of buffers.flags. */
#define BM_FLAG_TOPOLOGY_DIRTY 0
#define BM_FLAG_PAIR_DIRTY 1
#define BM_FLAG_PAIR_BUILDS 2
#define BM_FLAG_STEP 3           /* substep counter (history ping-pong parity) */
#define BM_FLAG_CANDIDATES 4     /* number of pair candidates */
#define BM_FLAG_EMBEDDED 5       /* count_embedded result */
#define BM_FLAG_SLOTS 6          /* registered slots */
#define BM_FLAG_CHANGED 7        /* entries of buffers.changed */
#define BM_FLAG_RELIST 8         /* entries of buffers.relist_list */
#define BM_FLAG_MULTI 9          /* entries of buffers.multi_nodes */
#define BM_FLAG_RELISTS 10       /* incremental pair-list updates run (codes changed, no full build) */
/* word 10 is unused */
#define BM_FLAG_MIXED_CELLS 11   /* entries of buffers.mixed_cells */
#define BM_FLAG_REGISTRATIONS 12 /* topology registrations run */
#define BM_FLAG_MAX_DISP 13      /* float bits: largest |x - ref| at the last full pair-list build */
#define BM_FLAG_HOLD_NEEDS 14    /* held-blade constraint: some contact violates this substep */
#define BM_FLAG_HOLD_RESIDUAL 15 /* float bits: largest final residual (m/s) of any constraint solve so far */
#define BM_FLAG_HOLD_COUNT 16    /* held-blade constraint: contacts this substep */
#define BM_FLAG_HOLD_NODES 17    /* held-blade constraint: grid nodes the contacts touch */
#define BM_FLAG_REG_MODE 18      /* this substep's registration: 0 none, 1 full, 2 incremental */
#define BM_FLAG_REG_CHANGED 19   /* entries of buffers.changed the incremental registration reads */
#define BM_FLAG_REG_NODES 20     /* entries of buffers.reg_nodes */
#define BM_FLAG_REG_CELLS 21     /* entries of buffers.reg_cells */
#define BM_FLAG_HOST_DIRTY 22    /* 1 after a host write that needs a full registration */
#define BM_FLAG_PAIR_SPEED 23    /* float bits: largest particle speed, found by a full pair-list build */
#define BM_FLAG_WORDS 24

typedef struct bm_solver bm_solver;
typedef struct bm_graph bm_graph;

/* Per-substep arguments of one batch of substeps (Solver._step_kernels,
 * solver.py:920-940). */
typedef struct bm_step_args {
    int32_t steps;         /* substeps in the batch */
    int32_t cut_bits;      /* BM_CUT_* bits, 0 when not cutting */
    int32_t cut_index;     /* digit of knife k is 3^(cut_index + k) */
    int32_t single_field;  /* transfers ignore cut codes (solver.py:382-389) */
    int32_t use_targets;   /* driven knife reads targets/rotations[i] */
    int32_t external_load; /* prepend load_external_state (coupling.py:118-131) */
    int32_t external_finish; /* append validate_interval + store_interval (coupling.py:132-136) */
    int32_t record_samples; /* 0, or samples of record_pose (coupling.py:139-147) */
    int32_t hold_pose;     /* record only first and last pose (hold mode) */
    int32_t pad;
} bm_step_args;

/* Size of the structs as compiled into the library (binding check). */
uint32_t bm_params_size(void);
uint32_t bm_buffers_size(void);
uint32_t bm_step_args_size(void);
const char* bm_last_error(void);
const char* bm_version(void);
/* Number of int32 words of buffers.scratch a solver with these params needs. */
int64_t bm_scratch_words(const bm_params* params);

/* Solver.__init__ (solver.py:157-316): checks the parameters and binds the buffers. */
int bm_solver_create(const bm_params* params, const bm_buffers* buffers, bm_solver** out);
int bm_solver_destroy(bm_solver* solver);

/* Solver.refresh_stress / material.compute_stress (solver.py:318-329, material.py:115-124). */
int bm_refresh_stress(bm_solver* s, void* stream);
/* Solver._register_topology (solver.py:391-429): (node, code) fields of every stencil node. */
int bm_register_topology(bm_solver* s, int single_field, void* stream);
/* Solver.material_step (solver.py:334-376): P2G, exchange, G2P + remap, F update. */
int bm_material_step(bm_solver* s, int single_field, void* stream);
/* Solver.rigid_contacts (solver.py:588-668): gravity, board and every knife. */
int bm_rigid_contacts(bm_solver* s, int cut_bits, void* stream);
/* Solver.particle_contacts (solver.py:670-751): pair contact with friction history. */
int bm_particle_contacts(bm_solver* s, void* stream);
/* BladeConstraint.solve (blade_constraint.py:254-324) for the externally held
 * knife 0 on the current grid velocities: the projected-gradient solve of the
 * broad-face contacts, its grid velocity correction and reaction.  Part of
 * every substep of an external tool in hold mode; exposed for tests. */
int bm_hold_constraint(bm_solver* s, void* stream);
/* bm_particle_contacts with the bucket-scan workspace of the pair-list rebuild
 * in a static device array of BM_STATIC_SCAN_PARTIALS ints (64 KiB) instead of
 * buffers.scratch; it allocates nothing.  No counterpart in the reference: it
 * serves hosts that step the contact pass inside their own frame loop under a
 * device-memory budget fixed at start-up, where an allocation would stall or
 * fail.  Limit: pair-list tables of at most 1024 * BM_STATIC_SCAN_PARTIALS
 * buckets (bucket_mask + 1), else BM_ERR_ARGUMENT.  The first call on each
 * device (the current one) looks up the array's address and should come
 * before any stream capture.  The address is kept for the life of the
 * process: after cudaDeviceReset (or any teardown of the device's primary
 * context) the library's device code may load elsewhere, so this entry point
 * must not be called again in that process.  Calls that overlap on one device (two streams,
 * solvers or host threads) share the array and race: serialise them.
 * Results equal bm_particle_contacts'. */
#define BM_STATIC_SCAN_PARTIALS 16384
int bm_particle_contacts_static(bm_solver* s, void* stream);
/* Solver.assign_sides (solver.py:866-890). */
int bm_assign_sides(bm_solver* s, int cut_index, int cutting, void* stream);
/* Solver._drive_tool (solver.py:824-864): targets/rotations row `index`. */
int bm_drive_tool(bm_solver* s, int index, void* stream);
/* Solver._finish_external_tool / _accumulate_tool_impulses (solver.py:788-822). */
int bm_finish_external(bm_solver* s, void* stream);
int bm_accumulate_tool_impulses(bm_solver* s, void* stream);
/* contact.clear_step (contact.py:1058-1068) for every knife. */
int bm_clear_step(bm_solver* s, void* stream);
/* One batch of substeps, launched eagerly on `stream`. */
int bm_substeps(bm_solver* s, const bm_step_args* args, void* stream);
/* The same batch captured once as a CUDA graph (Solver.prepare, solver.py:975-1019). */
int bm_graph_create(bm_solver* s, const bm_step_args* args, void* stream, bm_graph** out);
int bm_graph_launch(bm_graph* g, void* stream);
int bm_graph_destroy(bm_graph* g);
/* Batched sweeps: the batches of `count` independent solvers captured as one
 * CUDA graph, so one bm_graph_launch advances every instance (no reference
 * counterpart: the reference runs sweep instances one after another,
 * scripts/force_convergence.py:92-129).  Each solver's chain of kernels is an
 * independent branch; the chains are captured on `lanes` streams in the
 * given order (solver i on lane i % lanes), which sets how many run
 * concurrently.  args[i] are solver i's batch arguments. */
int bm_batch_graph_create(bm_solver* const* solvers, const bm_step_args* args, int count, int lanes, void* stream,
                          bm_graph** out);
/* Number of kernel launches one bm_graph_launch of `g` performs (its kernel nodes). */
int bm_graph_kernel_count(const bm_graph* g, int64_t* count);
/* diagnostics.Metrics.read (diagnostics.py:7-48) of the solver's state into
 * out[6] (device, float64): kinetic, gravitational and elastic energy (J),
 * largest speed (m/s), largest height z (m), smallest det F.  The sums are
 * exact before their one rounding to float64, so they do not depend on the
 * order of the particles; the extrema start from 0, -1e20 and 1e20. */
int bm_metrics(bm_solver* s, double* out, void* stream);
/* topology.components (topology.py:17-57) on the device.  codes: [n] cut
 * codes in device particle order, or NULL for the solver's codes; order: [n]
 * reference index of each device particle.  labels: [n] (by reference index)
 * piece of each particle, pieces ranked by their lowest reference index;
 * sizes: [n] particles per piece (the first *count entries); count: pieces,
 * or -1 if a union gave up.  All device pointers; labels and sizes are also
 * the workspace.  A stencil node joins a particle's piece when its float32
 * weight is positive. */
int bm_components(bm_solver* s, const int64_t* codes, const int64_t* order, int32_t* labels, int32_t* sizes,
                  int32_t* count, void* stream);
/* Nodal embedding of a surface in the deformed material (surface.py:825-993,
 * surface_gpu.py:11-345).  Reference nodes [node_count][3] and particle
 * reference positions [particle_count][3]; the support of node i is
 * indices/weights[offsets[i] .. offsets[i+1]) (tent weights, ascending
 * particle ids), extra_* the second ring (tent radius 2 h).  Floating arrays
 * hold doubles (scalar_bytes 8) or floats (4); all pointers are device
 * pointers, F is [n][9] row-major. */
typedef struct bm_embedding {
    int32_t node_count, particle_count, scalar_bytes, pad;
    const void* nodes;
    const void* reference;
    const int32_t* offsets;
    const int32_t* indices;
    const void* weights;
    const int32_t* extra_offsets; /* may be NULL when extend == 0 */
    const int32_t* extra_indices;
    const void* extra_weights;
} bm_embedding;
/* MaterialEmbedding.field / node_state (surface.py:936-963): positions
 * [node_count][3] and gradients [node_count][9] of each node's field for
 * node_codes[i] (or `code` when node_codes is NULL); NaN where no compatible
 * particle supports the node; with `extend` the second ring serves nodes the
 * first cannot, and *extensions counts them (added to its value). */
int bm_embed_nodes(const bm_embedding* e, const void* x, const void* F, const int64_t* codes,
                   const int64_t* node_codes, int64_t code, int extend, void* positions, void* gradients,
                   int32_t* extensions, void* stream);
/* MaterialEmbedding.vertices through a material grid (surface_gpu.py:270-345):
 * vertex v = sum_k corner_weights[v][k] * field(vertex_codes[v]) at node
 * corners[v][k] (second ring allowed).  counts[0] += extended corner lookups,
 * counts[1] += corners with weight > 1e-9 and no support (an error). */
int bm_embed_vertices(const bm_embedding* e, int vertex_count, const int64_t* vertex_codes, const int32_t* corners,
                      const void* corner_weights, const void* x, const void* F, const int64_t* codes, void* vertices,
                      int32_t* counts, void* stream);
/* TopoCut topology discovery for the MLS baseline (topocut_topology.py:31-229).
 * Voxel points (i, j, k) sit at lower + voxel * (i, j, k), dims[] per axis,
 * values stored row-major [dims0][dims1][dims2].  Particles are binned in
 * cubes of edge `reach` (bin_dims[] of them from `lower`).  poses: [pose_count]
 * knife poses of the carved trajectory, 7 floats each (position, quaternion
 * xyzw), half: the knife half extents.  Device pointers throughout. */
typedef struct bm_topocut_grid {
    int32_t dims[3], bin_dims[3];
    float lower[3], voxel, radius, reach, half[3];
    int32_t pose_count;
    const float* poses;
} bm_topocut_grid;
/* particle_sdf (topocut_topology.py:39-64): field = max(min |v - x_p| - radius,
 * -v_z) over particles within reach, raised to one voxel inside any carved
 * knife box.  x: [n][3].  Workspace: bin_start [bins + 1], bin_fill [bins],
 * items [n], partials [bins / 1024 + 1], ticket [1] (zero). */
int bm_topocut_sdf(const bm_topocut_grid* g, const float* x, int n, float* field, int32_t* bin_start,
                   int32_t* bin_fill, int32_t* items, int32_t* partials, int32_t* ticket, void* stream);
/* Zero isosurface of `field` (value < 0 inside) by marching tetrahedra, first
 * pass: triangles per cube (cube_tris, tri_start = their exclusive scan,
 * [cubes]) and crossed lattice edges (edge_used, edge_index = vertex index,
 * [points * 7]); totals[0] triangles, totals[1] vertices.  partials holds
 * points * 7 / 1024 + 1 ints. */
int bm_topocut_count(const bm_topocut_grid* g, const float* field, int32_t* cube_tris, int32_t* tri_start,
                     int32_t* edge_used, int32_t* edge_index, int32_t* partials, int32_t* ticket, int32_t* totals,
                     void* stream);
/* Second pass: vertices [totals[1]][3] and triangles [totals[0]][3], each
 * oriented from the inside to the outside; vertices are shared along edges. */
int bm_topocut_emit(const bm_topocut_grid* g, const float* field, const int32_t* tri_start, const int32_t* edge_used,
                    const int32_t* edge_index, float* vertices, int32_t* triangles, void* stream);
/* nearest_cluster (topocut_topology.py:67-78): labels[p] = the mesh (triangles
 * mesh_start[m] .. mesh_start[m+1]) with the smallest signed distance to x_p
 * below tau (negative inside by winding number; meshes farther than reach are
 * skipped), else -1. */
int bm_topocut_cluster(const float* x, int n, const float* vertices, const int32_t* triangles,
                       const int32_t* mesh_start, int mesh_count, float tau, float reach, int32_t* labels,
                       void* stream);
/* Stages of one substep, in launch order (profiling). */
#define BM_STAGE_PROLOGUE 0  /* clear_pair_slots + clear_step */
#define BM_STAGE_RIGID 1     /* rigid_and_speed + extra_blade */
#define BM_STAGE_PAIRS 2     /* pair list rebuild (when needed) + pairs_listed */
#define BM_STAGE_REGISTER 3  /* _register_topology (when needed) */
#define BM_STAGE_P2G 4       /* p2g + couple_and_velocity */
#define BM_STAGE_G2P 5       /* g2p of g2p_remap */
#define BM_STAGE_REMAP 6     /* remap scatter + couple */
#define BM_STAGE_TOOL 7      /* tool.step / finish_external_step */
#define BM_STAGE_FUPDATE 8   /* update_F + stress */
#define BM_STAGE_ASSIGN 9    /* contact.assign (side labels) */
#define BM_STAGES 10

/* The batch of bm_substeps launched eagerly with a CUDA event pair around
 * every stage; stage_ms[BM_STAGES] receives the summed device time of each
 * stage over the batch (the host waits after every substep).  Results are
 * identical to bm_substeps. */
int bm_substeps_profiled(bm_solver* s, const bm_step_args* args, float* stage_ms, void* stream);

/* contact.count_embedded (contact.py:1042-1055) into flags[BM_FLAG_EMBEDDED]. */
int bm_count_embedded(bm_solver* s, int reset, void* stream);
/* material.validate_interval (material.py:6-20). */
int bm_validate_interval(bm_solver* s, void* stream);
/* Convert the 128-bit accumulators to float32 API arrays:
 * reaction [tools][3], torque [tools][3], board [3], work [1]. */
int bm_read_accumulators(bm_solver* s, float* reaction, float* torque, float* board, float* work, void* stream);
/* Overwrite the accumulators from float32 API arrays (any may be NULL). */
int bm_write_accumulators(bm_solver* s, const float* reaction, const float* torque, const float* board,
                          const float* work, void* stream);
/* Write the tool float32 mirror from the float64 tool state (after host writes). */
int bm_sync_tool_mirror(bm_solver* s, void* stream);

/* Kernel-level entry points on caller buffers, used by unit tests and by
 * callers of the reference's @wp.func helpers. */
/* contact.blade_query (contact.py:46-120), n points (AoS float3). */
int bm_blade_query(const float* local, int n, const float* half, float bevel, float* closest, float* normal,
                   float* distance, void* stream);
/* contact.friction (contact.py:21-43), normal/relative/history AoS float3 [n]. */
int bm_friction(const float* normal, const float* relative, const float* jn, const float* history, int n, float me,
                float dt, float mus, float mud, float gk, float gc, float* impulse, float* new_history, void* stream);
/* material.couple over explicit node lists (material.py:155-193): fields are
 * given per node as runs in `order` (ascending code), AoS float3 state. */
int bm_couple_fields(const int64_t* codes, const float* mass, const float* state, const int32_t* node_start,
                     int nodes, float* result, void* stream);
/* material.g2p (material.py:343-381) on explicit slots/weights (AoS float3). */
int bm_g2p_probe(float* x, float* v, const int32_t* slots, const float* weights, const float* old_v,
                 const float* new_v, int n, float dt, float flip, void* stream);
/* contact.resist_cut (contact.py:181-232) for n particles (AoS float3 inputs). */
int bm_resist_cut_probe(const float* j, const float* x, const float* v, const float* origin,
                        const float* tool_velocity, const float* q, const float* tool_angular, const float* half,
                        float radius, float spacing, float* damage, float threshold, int cutting, uint64_t* work_acc,
                        float* result, int n, void* stream);
/* material.plastic_project (material.py:434-442) on [9][n] F and Fp. */
int bm_plastic_project(float* F, float* Fp, int n, float mu, float yield_stress, int32_t* errors, void* stream);
/* Accuracy probes of the library's own arithmetic beside CUDA's.  No
 * counterpart in the reference, which calls Warp's builtins (wp.log, wp.exp,
 * wp.sin, wp.cos, wp.atan2, wp.svd3 at material.py:111,418,515,565,588 and
 * tool.py:178-259); these measure the replacements.  bm_math_probe_f: kind
 * 0 logf, 1 expf, 2 expm1f of x[i]; out[2i] = the library's, out[2i+1] =
 * CUDA's.  bm_math_probe_d (float64): kind 0 sin, 1 cos of x[i], 2
 * atan2(y[i], x[i]).  bm_svd_probe: row-major 3x3 matrices A[n] to
 * U diag(sigma) V^T (the substep's SVD) and the polar rotation R. */
int bm_math_probe_f(int kind, const float* x, int n, float* out, void* stream);
int bm_math_probe_d(int kind, const double* x, const double* y, int n, double* out, void* stream);
int bm_svd_probe(const float* A, int n, float* U, float* sigma, float* V, float* R, void* stream);

/* ------------------------------------------------------------------------
 * MLS-MPM cutting baseline (blademaster_warp/mlsmpm.py): updated-Lagrangian
 * MLS-MPM with quadratic B-splines, APIC transfer and one velocity field on
 * a dense grid, TopoCut damage (Eqs. 6-7), and the same rigid contact as the
 * TLMPM solver with knife 0 held (tool model -1, zero mobility).  Particles
 * stay in the reference order.  Grid sums are exact 64-bit fixed point
 * (value * 2^shift), so they do not depend on the order of the scatter.
 * ------------------------------------------------------------------------ */
typedef struct bm_mls_params {
    int32_t n;
    int32_t dims[3];          /* dense grid nodes per axis */
    int32_t plastic;          /* yield_stress > 0: Hencky return map with softening */
    int32_t mass_shift;       /* grid mass fixed point: value * 2^mass_shift */
    int32_t momentum_shift;   /* grid momentum fixed point: value * 2^momentum_shift */
    int32_t pad;
    float origin[3];          /* position of grid node (0, 0, 0) */
    float dx, dt, mass, volume, mu, lam;
    float damaged_shear;      /* shear modulus factor of damaged particles */
    float softening;          /* Eq. 7 gamma, Pa per unit plastic strain */
    float compressed, stretched; /* Eq. 6 J bounds */
} bm_mls_params;

typedef struct bm_mls_buffers {
    float* x;                 /* [3][n] reference particle order */
    float* v;                 /* [3][n] */
    float* C;                 /* [9][n] APIC affine velocity, row-major */
    float* F;                 /* [9][n] */
    float* yield_stress;      /* [n] */
    float* damage;            /* [n] */
    float* damage_reference;  /* [n] J of the Eq. 6 reference state, 0 while damage is off */
    int64_t* grid_mass;       /* [nodes] fixed point */
    int64_t* grid_momentum;   /* [3][nodes] fixed point */
    float* grid_v;            /* [3][nodes] */
    int32_t* inversions;      /* [1] particle-steps with det F <= 0 before the clamp */
} bm_mls_buffers;

typedef struct bm_mls bm_mls;

/* MlsSolver.__init__ (mlsmpm.py:232-291).  `contact` and `contact_buffers`
 * describe the rigid contact exactly as for bm_solver_create (n and the
 * particle arrays x, v shared with `buffers`; one tool; histories [2][3][n],
 * hist_mask, damage [n] unused, impulses [3][n], tool, tool_f, mobility, acc,
 * interval, speed, errors, flags, packed, result). */
int bm_mls_create(const bm_mls_params* params, const bm_mls_buffers* buffers, const bm_params* contact,
                  const bm_buffers* contact_buffers, bm_mls** out);
int bm_mls_destroy(bm_mls* s);
/* `steps` substeps (MlsSolver._substep, mlsmpm.py:293-393) after loading the
 * knife state from contact_buffers.packed (load_external_state). */
int bm_mls_substeps(bm_mls* s, int steps, void* stream);
/* The same interval captured as a CUDA graph (MlsSolver.advance, mlsmpm.py:395-426). */
int bm_mls_graph_create(bm_mls* s, int steps, void* stream, bm_graph** out);

/* ------------------------------------------------------------------------
 * Learned tool predictor (no reference counterpart: it stands in for the
 * linear mobility prediction of tool_substep "predict", tool.py:97-113).
 * ------------------------------------------------------------------------ */
/* Test hook: the poll limit of bm_gemm_tn_bf16's waits inside its K loop
 * on the current device (limit < 0 restores the default).  With 0 the first
 * wait for a stage gives up at once, so a GEMM of K >= 128 records status 1
 * after draining the MMAs in flight (the drain always waits the full limit);
 * tests use it to drive the timeout path. */
int bm_gemm_set_loop_wait_limit(long long limit);
/* D[M x N] = A[M x K] * B[N x K]^T on the tensor cores (tcgen05): A and B
 * bf16, row-major (K contiguous), fp32 accumulation, then + bias[N] and ReLU
 * if requested; D (fp32) and/or D_bf16 receive the result.  N in 16..256 (a
 * multiple of 16), K a multiple of 32, A, B and D 16-byte aligned, D_bf16
 * 8-byte aligned (BM_ERR_ARGUMENT otherwise).  *status is
 * set to 1 if the tensor-core work did not complete in time. */
int bm_gemm_tn_bf16(const uint16_t* A, const uint16_t* B, float* D, int M, int N, int K, const float* bias, int relu,
                    uint16_t* D_bf16, int32_t* status, void* stream);
/* Training kernels of the predictor: bf16 transpose ([rows x cols] -> [cols x rows]),
 * ReLU backward (g * (h > 0) to bf16), mean-squared-error gradient over `outputs`
 * of `width` stored columns (adds the loss to *loss), column sums, fp32 -> bf16
 * with a padded row pitch, and one Adam step (bias-corrected, step >= 1). */
int bm_mlp_transpose16(const uint16_t* in, uint16_t* out, int rows, int cols, void* stream);
int bm_mlp_relu_grad(float* g, const uint16_t* h, uint16_t* out, int64_t count, void* stream);
/* Predictor input: particle counts of 4 x 4 x 4 bins in the frame of knife 0
 * (tool_f, one BM_TOOL_F_WORDS record) around its edge, x in [-4h, 4h) across
 * the blade, y in [-half_y, half_y), z in [-4h, 4h) about the edge;
 * x is [3][n]; counts[64] are overwritten. */
int bm_mlp_pool(const float* x, int n, const float* tool_f, float h, float half_y, int32_t* counts, void* stream);
int bm_mlp_mse_grad(const float* y, const float* t, int rows, int outputs, int width, float* d, uint16_t* d_bf16,
                    float* loss, void* stream);
int bm_mlp_colsum(const float* g, int rows, int cols, float* out, void* stream);
int bm_mlp_cast_bf16(const float* x, int rows, int cols, int pitch, uint16_t* out, void* stream);
int bm_mlp_adam(float* w, const float* g, float* m, float* v, uint16_t* w_bf16, int64_t count, float lr, float beta1,
                float beta2, float eps, int step, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* BLADEMASTER_GB300_H */
