/*
 * lfgpu.h — C ABI of the GB300-native LightFEM solve path (liblfgpu.so).
 *
 * Plain C: opaque handle, int32 status returns, caller-owned HOST buffers, no
 * exceptions and no torch or CUDA types across the boundary.  One handle owns one
 * CUDA stream and its device buffers; a handle is not thread-safe, distinct
 * handles are independent.  Every entry point returns LFGPU_OK (0) or an
 * lfgpu_status code; lfgpu_last_error() gives the message.
 *
 * The entry points replace these internal seams of the reference host library
 * (paths relative to the LightFEM source tree):
 *
 *   lfgpu_set_mesh / lfgpu_set_pattern / lfgpu_set_loads / lfgpu_assemble
 *        assemble(const Model&) -> AssembledSystem        src/solver.cpp:219-334
 *        (q4_stiffness src/element.cpp:130-161, coloring_assembly / atomic_assembly
 *         src/solver.cpp:144-179, loads src/solver.cpp:303-332)
 *   lfgpu_apply_dirichlet
 *        apply_dirichlet(...)                              src/solver.cpp:355-413
 *        + the zero-pivot sweep                            src/solver.cpp:920-940
 *   lfgpu_solve
 *        solve_iterative(...) -> LinearSolverReport       src/solver.cpp:675-747
 *        (pcg_solve src/solver.cpp:532-627, BsrMatrix src/sparse.cpp:128-204,
 *         JacobiPreconditioner src/solver.cpp:497-509, SubdomainBlockJacobi with
 *         one node per subdomain src/precond.cpp:121-291, IncompleteCholesky0
 *         src/precond.cpp:298-412)
 *   lfgpu_reactions
 *        reaction = K_full u - f                           src/solver.cpp:953-954
 *   lfgpu_postprocess
 *        postprocess + smooth_nodal_stresses               src/solver.cpp:756-871
 *
 * Error mapping to the reference's exceptions (src/main.cpp:162-164 maps all of them
 * to exit code 4): LFGPU_ERR_JACOBIAN -> "Q4 stiffness evaluation received a
 * non-positive Jacobian" (src/element.cpp:52-54); LFGPU_ERR_NOT_SPD -> "PCG
 * encountered non-positive curvature; system is not SPD" (src/solver.cpp:591-593);
 * LFGPU_ERR_RHO_INITIAL / LFGPU_ERR_RHO -> src/solver.cpp:579-581 / :616-618;
 * LFGPU_ERR_MECHANISM -> src/solver.cpp:926-936; a report with converged == 0
 * -> "PCG did not converge" (src/solver.cpp:948-950).
 */
#ifndef LFGPU_H
#define LFGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct lfgpu_context* lfgpu_t;

typedef enum lfgpu_status {
    LFGPU_OK = 0,
    LFGPU_ERR_ARGUMENT = 1,        /* bad size, index or option (std::invalid_argument) */
    LFGPU_ERR_CUDA = 2,            /* a CUDA runtime call failed */
    LFGPU_ERR_STATE = 3,           /* call order violated (std::logic_error) */
    LFGPU_ERR_JACOBIAN = 4,        /* an element has detJ <= 1e-14 at a Gauss point */
    LFGPU_ERR_EDGE = 5,            /* zero-length loaded edge */
    LFGPU_ERR_MECHANISM = 6,       /* zero pivot carrying load */
    LFGPU_ERR_NOT_SPD = 7,         /* p.Kp <= 0 or non-finite */
    LFGPU_ERR_RHO_INITIAL = 8,     /* r0.z0 <= 0 or non-finite */
    LFGPU_ERR_RHO = 9,             /* r.z <= 0 or non-finite during the iteration */
    LFGPU_ERR_NONFINITE_DIAG = 10, /* non-finite diagonal in the Jacobi setup */
    LFGPU_ERR_TIMEOUT = 11,        /* a device-side wait exceeded its bound */
    LFGPU_ERR_NOMEM = 12,          /* device allocation failed */
    LFGPU_ERR_UNSUPPORTED = 13,    /* option combination not built */
    LFGPU_ERR_SCRATCH_LIMIT = 14   /* system larger than LFGPU_NOALLOC_MAX_ROWS */
} lfgpu_status;

enum { LFGPU_PLANE_STRESS = 0, LFGPU_PLANE_STRAIN = 1 };
enum { LFGPU_ASSEMBLY_COLORING = 0, LFGPU_ASSEMBLY_ATOMIC = 1 };
enum { LFGPU_STORAGE_CSR = 0, LFGPU_STORAGE_BSR = 1 };
/* BLOCK2: the 2x2 nodal case (subdomain_nodes 1) fused into the loop kernels.
 * SUBDOMAIN: SubdomainBlockJacobi with the handle's lfgpu_set_subdomains split
 * (the reference's `preconditioner block` with any subdomain_nodes). */
enum { LFGPU_PRECOND_JACOBI = 0, LFGPU_PRECOND_BLOCK2 = 1, LFGPU_PRECOND_IC0 = 2, LFGPU_PRECOND_SUBDOMAIN = 3 };
enum { LFGPU_SPLIT_RCB = 0, LFGPU_SPLIT_CHUNK = 1 };
enum { LFGPU_PRECISION_FP64 = 0, LFGPU_PRECISION_MIXED = 1 };
enum { LFGPU_REFINE_RELIABLE = 0, LFGPU_REFINE_RESTART = 1 };
enum { LFGPU_EDGE_TRACTION = 0, LFGPU_EDGE_PRESSURE = 1 };
/* Handle options (lfgpu_set_option). */
enum {
    LFGPU_OPTION_WAIT_LIMIT_NS = 0, /* how long a bounded device-side wait spins before it gives up with
                                       LFGPU_ERR_TIMEOUT (default 4e9 ns); tests shorten it */
    LFGPU_OPTION_IC0_SWEEP = 1      /* LFGPU_IC0_SWEEP_*: how the IC(0) triangular sweeps are scheduled */
};
/* AUTO: by levels (one thread-block cluster walks the dependency levels) when the
 * pattern's level schedule fits the cluster's shared-memory ring and its levels
 * hold 192 rows or more on average, else POLLED.  The mixed-precision loop always
 * sweeps by levels.
 * LEVELS: by levels, LFGPU_ERR_UNSUPPORTED where the schedule does not fit.
 * POLLED: row chunks in sweep order, each row polling for its operands (FP64 only). */
enum { LFGPU_IC0_SWEEP_AUTO = 0, LFGPU_IC0_SWEEP_LEVELS = 1, LFGPU_IC0_SWEEP_POLLED = 2 };

/* Arrays lfgpu_download can return. */
enum {
    LFGPU_K_FULL = 0,        /* nnz: assembled K before Dirichlet (AnalysisResult::stiffness) */
    LFGPU_K_CONSTRAINED = 1, /* nnz: K after elimination and the zero-pivot sweep */
    LFGPU_F_FULL = 2,        /* n: assembled load vector (AnalysisResult::load) */
    LFGPU_F_CONSTRAINED = 3, /* n: right-hand side after elimination */
    LFGPU_U = 4,             /* n: last solution */
    LFGPU_R = 5              /* n: last reactions */
};

typedef struct lfgpu_solve_options {
    double tolerance;          /* stop when ||r|| <= tolerance * max(1, ||f||) */
    int64_t max_iterations;    /* PCG iteration cap (inner iterations for mixed) */
    int32_t storage;           /* LFGPU_STORAGE_* */
    int32_t preconditioner;    /* LFGPU_PRECOND_* */
    int32_t precision;         /* LFGPU_PRECISION_* */
    int32_t refinement;        /* LFGPU_REFINE_* (mixed only) */
    double inner_reduction;    /* mixed: FP32 residual drop that triggers an FP64 update */
    int64_t max_refinements;   /* mixed: cap on FP64 residual replacements */
    int32_t persistent;        /* 1: one persistent cooperative kernel; 0: device-driven CUDA graph of
                                  per-phase kernels (conditional WHILE node) */
    int32_t unrolled;          /* profiling only, graph loop: > 0 replaces the conditional loop by a plain
                                  graph of this many iterations (profilers do not descend into
                                  conditional bodies); the solve stops there */
} lfgpu_solve_options;

/* Mirrors LinearSolverReport (include/lightfem/solver.hpp:12-34) plus GPU fields. */
typedef struct lfgpu_report {
    int32_t converged;
    int32_t status;                  /* lfgpu_status of the solve */
    int64_t iterations;              /* PCG iterations (FP32 inner iterations for mixed) */
    int64_t refinements;             /* mixed: FP64 residual replacements */
    double initial_residual;         /* ||f|| */
    double final_residual;           /* FP64 PCG: recursive ||r||; mixed: true FP64 ||f - K u|| */
    double true_residual;            /* ||f - K u|| recomputed in FP64 after the solve */
    double solve_ms;                 /* device time of the solve (CUDA events) */
    double matvec_ms;                /* device time of one standalone SpMV x matvec_calls */
    int64_t matvec_calls;
    int64_t matrix_bytes_per_matvec; /* bytes of the matrix one product streams (int32 columns; mixed BSR:
                                        16-bit column offsets when they fit; mixed CSR of a paired
                                        pattern: the BSR blocks, its FP32 working copy) */
    double storage_convert_ms;       /* CSR -> BSR conversion this solve ran (BSR storage; mixed CSR of a
                                        paired pattern) */
    double preconditioner_setup_ms;
    double preconditioner_apply_ms;  /* IC0 only: device time of the triangular sweeps */
    int64_t subdomains;              /* block / subdomain: number of subdomains (2x2 nodal blocks for block) */
    double capture_ratio;            /* block / subdomain: share of nonzeros inside a subdomain */
    int64_t degenerate_subdomains;   /* block / subdomain: blocks that fell back to the identity */
    int64_t ic0_breakdowns;          /* ic0: clamped pivots */
    int64_t ic0_levels;              /* ic0: forward + backward level count */
    int64_t fallback_fp64;           /* mixed: 1 if the FP32 inner solve stagnated and FP64 PCG finished */
    /* Persistent kernel: time as CTA 0 sees it, summed over iterations: [0] product
     * phase, [1] grid sum after it, [2] update phase, [3] grid sum after it, [4] FP64:
     * p update / mixed: residual replacements, [5] FP64: barrier after the p update.
     * Profiling run (unrolled > 0, up to 5000 passes): device time of each kernel
     * kind summed over the passes (CUDA events between launches): [0] product,
     * [1] update, [2] FP64 p update / mixed residual replacement / IC(0) forward
     * sweep, [3] mixed re-preconditioning / IC(0) backward sweep, [4] IC(0) r.z,
     * [5] IC(0) p update.  Graph runs leave it zero.  matvec_ms equals phase_ms[0]. */
    double phase_ms[6];
} lfgpu_report;

/* Stage timings of the last calls (device time, CUDA events), as in PerformanceReport. */
typedef struct lfgpu_timings {
    double pattern_ms;       /* lfgpu_build_pattern */
    double assembly_ms;      /* element stiffness + scatter + element loads */
    double boundary_ms;      /* retain copy + elimination + zero-pivot sweep */
    double reactions_ms;
    int64_t coloring_count;  /* colours used by the colouring strategy */
    int64_t kernel_launches; /* kernels this handle has launched so far (graph nodes included) */
    double postprocess_ms;   /* element fields + nodal smoothing (lfgpu_postprocess) */
    double rcm_ms;           /* lfgpu_rcm (host wall time, device work included) */
    double adjoint_kernel_ms; /* lfgpu_adjoint: the gradient kernel alone (no solve, no download) */
} lfgpu_timings;

/* --- handle ------------------------------------------------------------------- */
int lfgpu_create(int device, lfgpu_t* out);
int lfgpu_destroy(lfgpu_t h);
const char* lfgpu_last_error(lfgpu_t h);
const char* lfgpu_version(void);
/* The last failure a kernel of this handle reported, for hosts that rebuild the
 * reference's message from their own model: *status its lfgpu_status (0: none so
 * far), *index the element index (LFGPU_ERR_JACOBIAN, LFGPU_ERR_EDGE), DOF
 * (LFGPU_ERR_MECHANISM) or CTA (LFGPU_ERR_TIMEOUT) it names.  For
 * LFGPU_ERR_MECHANISM values[0] and values[1] receive the DOF's constrained load
 * and diagonal, the two numbers the zero-pivot exception prints
 * (src/solver.cpp:926-936); for LFGPU_ERR_TIMEOUT values[0] is 1 when the wait
 * raised the abort flag that stops every other wait; otherwise both are 0.  Any
 * pointer may be NULL. */
int lfgpu_failure_detail(lfgpu_t h, int32_t* status, int64_t* index, double* values);
/* Set a handle option (LFGPU_OPTION_*).  No reference counterpart: the reference
 * has no device waits and sweeps serially. */
int lfgpu_set_option(lfgpu_t h, int32_t option, int64_t value);

/* --- model -------------------------------------------------------------------- */
/* Nodes in index order (node k owns DOFs 2k, 2k+1: Model::rebuild_indices,
 * src/model.cpp:80-84), Q4 elements as node indices in counter-clockwise order,
 * one material index per element into (young, poisson, thickness).
 * Replaces the per-element inputs of q4_stiffness (src/element.cpp:130-161). */
int lfgpu_set_mesh(lfgpu_t h, int64_t n_nodes, const double* xy, int64_t n_elements,
                   const int32_t* element_nodes, const int32_t* element_material,
                   int64_t n_materials, const double* young, const double* poisson,
                   const double* thickness, int32_t plane_mode);

/* Replace the moduli of the material table (used by the adjoint loop). */
int lfgpu_set_young(lfgpu_t h, const double* young);

/* CSR pattern and element->value map as build_csr_assembly_pattern produces them
 * (src/sparse.cpp:15-58): row_offsets[n+1], columns[nnz] ascending per row with the
 * diagonal present, element_value_index[64 E] row-major per element, and the colour
 * of every element (element_colors, src/solver.cpp:100-133; NULL if only the atomic
 * strategy will be used). */
int lfgpu_set_pattern(lfgpu_t h, int64_t n_dofs, int64_t nnz, const int64_t* row_offsets,
                      const int32_t* columns, const int32_t* element_value_index,
                      const int32_t* element_color);

/* Build the pattern, map and colouring of the current mesh inside the library
 * (same output as build_csr_assembly_pattern + element_colors). */
int lfgpu_build_pattern(lfgpu_t h);
int lfgpu_pattern_info(lfgpu_t h, int64_t* n_dofs, int64_t* nnz, int64_t* n_colors);
int lfgpu_download_pattern(lfgpu_t h, int64_t* row_offsets, int32_t* columns,
                           int32_t* element_value_index, int32_t* element_color);

/* Loads (src/solver.cpp:303-332).  nodal[n] holds the summed nodal loads (may be
 * NULL); body force and edge load records refer to element indices; edge_side is the
 * Q4 local edge 1..4, edge_kind LFGPU_EDGE_*, edge_first = tx or pressure,
 * edge_second = ty. */
int lfgpu_set_loads(lfgpu_t h, const double* nodal, int64_t n_body, const int32_t* body_element,
                    const double* body_bx, const double* body_by, int64_t n_edge,
                    const int32_t* edge_element, const int32_t* edge_side,
                    const int32_t* edge_kind, const double* edge_first,
                    const double* edge_second);

/* Prescribed displacements, sorted or not (collect_constraints, src/solver.cpp:340-351). */
int lfgpu_set_constraints(lfgpu_t h, int64_t count, const int64_t* dofs, const double* values);

/* --- the solve path ----------------------------------------------------------- */
int lfgpu_assemble(lfgpu_t h, int32_t strategy);
int lfgpu_apply_dirichlet(lfgpu_t h);
/* u_out may be NULL (the solution stays on the device). */
int lfgpu_solve(lfgpu_t h, const lfgpu_solve_options* options, double* u_out, lfgpu_report* report);
/* R = K_full u - f_full for the last solution; r_out may be NULL. */
int lfgpu_reactions(lfgpu_t h, double* r_out);

/* Post-processing of the last solution: postprocess + smooth_nodal_stresses
 * (src/solver.cpp:756-871, q4_center_field / q4_gauss_point_fields
 * src/element.cpp:212-248).  element_fields[35 e + 7 k + j] (may be NULL): k = 0
 * the element centre, k = 1..4 the Gauss points (-g,-g), (g,-g), (g,g), (-g,g);
 * j = strain xx, yy, xy, stress xx, yy, xy, von Mises.  nodal_stress[4 i + j]
 * (may be NULL): smoothed stress xx, yy, xy and its von Mises, zero for a node in
 * no element. */
int lfgpu_postprocess(lfgpu_t h, double* element_fields, double* nodal_stress);
int lfgpu_download(lfgpu_t h, int32_t which, double* out);
int lfgpu_timings_get(lfgpu_t h, lfgpu_timings* out);

/* Device timing across several calls: record event `slot` (0..7) on the handle's
 * stream, and read the device time between two recorded slots (synchronises). */
int lfgpu_event_record(lfgpu_t h, int32_t slot);
int lfgpu_event_elapsed(lfgpu_t h, int32_t slot_a, int32_t slot_b, double* ms);

/* One product y = A x on the device copy of K_CONSTRAINED (which = 1) or K_FULL
 * (which = 0) in the given storage and precision; device-timed over `repeat` calls.
 * Used by the tests and to report SpMV bandwidth. */
int lfgpu_spmv(lfgpu_t h, int32_t which, int32_t storage, int32_t precision, const double* x,
               double* y, int32_t repeat, double* ms_per_call);

/* Subdomains of the SUBDOMAIN preconditioner (build_dof_subdomain,
 * src/solver.cpp:631-653): nodes_per_subdomain nodes each, split LFGPU_SPLIT_RCB
 * (split_by_coordinates, src/precond.cpp:30-105) or LFGPU_SPLIT_CHUNK
 * (split_by_chunks, :19-28) over the node order of lfgpu_set_mesh.  The defaults
 * are the reference's (64, RCB; include/lightfem/model.hpp:107-108).  RCB pieces
 * can hold up to about twice the requested nodes.  One CTA factors and solves a
 * subdomain, a thread per DOF, so a subdomain holds at most
 * LFGPU_SUBDOMAIN_MAX_DOFS DOFs; a larger one makes the solve return
 * LFGPU_ERR_UNSUPPORTED. */
#define LFGPU_SUBDOMAIN_MAX_DOFS 1024
int lfgpu_set_subdomains(lfgpu_t h, int64_t nodes_per_subdomain, int32_t split);

/* One FP64 application z = M^-1 r of a preconditioner of K_CONSTRAINED, built on
 * first use: JacobiPreconditioner::apply (src/solver.cpp:497-509), the 2x2 nodal
 * or the general SubdomainBlockJacobi::apply (src/precond.cpp:242-291) or
 * IncompleteCholesky0::apply (src/precond.cpp:386-412).  *ms (may be NULL) gets the
 * device time of the application. */
int lfgpu_apply_preconditioner(lfgpu_t h, int32_t preconditioner, const double* r, double* z,
                               double* ms);

/* --- sensitivities (no reference counterpart) ---------------------------------- */
/* Gradient of J(u) with respect to the modulus of every element's material entry,
 * scaled per element: grad[e] = -lambda_e^T K_e u_e / E_e, with K lambda = dJ/du
 * (dJ/du zeroed on constrained DOFs).  dj_du == NULL means compliance J = f.u, for
 * which lambda = u and no second solve runs.  Uses the last solution. */
int lfgpu_adjoint(lfgpu_t h, const double* dj_du, const lfgpu_solve_options* options,
                  double* grad, lfgpu_report* report);

/* --- allocation-free residual norm (no reference counterpart) ------------------ */
/* The reference has no counterpart: it never runs on a device.  *norm_out =
 * ||f - K u||_2 for a CSR system held in the CALLER's device memory (row_offsets
 * int32[n_rows + 1], columns int32[nnz], values double[nnz], u and f double[n_rows];
 * device pointers, current device), the residual lfgpu_solve reports as
 * true_residual.  It allocates nothing: for callers that cannot allocate device
 * memory (frameworks whose pool owns all device memory, loops where an
 * allocation's implicit synchronisation is not acceptable).  Its only scratch is
 * a fixed 512 KiB static device array, so n_rows <= LFGPU_NOALLOC_MAX_ROWS;
 * larger systems return LFGPU_ERR_SCRATCH_LIMIT.  The first call on a device (and
 * the first in each new context on it) resolves the array's address with that
 * device current, which may load the module there: make it before any stream
 * capture.  All calls in a context share the array, which keeps the last call's
 * contents; calls that overlap on the GPU (two streams or two threads) race on
 * it.  Runs on `stream` (NULL: the legacy default stream), copies the norm to
 * *norm_out and synchronises `stream` before it returns. */
#define LFGPU_NOALLOC_MAX_ROWS 4194304
int lfgpu_residual_norm_noalloc(int64_t n_rows, const int32_t* row_offsets, const int32_t* columns,
                                const double* values, const double* u, const double* f, void* stream,
                                double* norm_out);

/* Reverse Cuthill-McKee order of the handle's mesh (reverse_cuthill_mckee,
 * src/reordering.cpp:11-62), computed on the device: order_out[n_nodes] receives
 * node indices of the mesh given to lfgpu_set_mesh.  The reference ranks ties by
 * node ID, so pass the nodes in ascending-ID order to get the reference's order. */
int lfgpu_rcm(lfgpu_t h, int64_t* order_out);

/* csr_profile (src/sparse.cpp:227-242) of the CSR pattern the handle's mesh
 * produces, without building it: profile_out[4] = {dimension, nonzeros, bandwidth,
 * profile}.  The reference reports it before and after RCM
 * (PerformanceReport::before / after, src/solver.cpp:886-898). */
int lfgpu_mesh_profile(lfgpu_t h, int64_t* profile_out);

/* --- host utilities (setup the reference performs on the host) ----------------- */
/* reverse_cuthill_mckee (src/reordering.cpp:11-62): node IDs in the new order. */
int lfgpu_host_rcm(int64_t n_nodes, const int64_t* node_ids, int64_t n_elements,
                   const int64_t* element_node_ids, int64_t* order_out);
/* split_by_chunks / split_by_coordinates (src/precond.cpp:19-105): subdomain of
 * every node (owner_out[n_nodes]) and the subdomain count; xy holds 2 coordinates
 * per node.  The split lfgpu_set_subdomains uses. */
int lfgpu_host_subdomains(int64_t n_nodes, const double* xy, int64_t nodes_per_subdomain, int32_t split,
                          uint32_t* owner_out, int64_t* count_out);

#ifdef __cplusplus
}
#endif

#endif /* LFGPU_H */
