// Launchers each kernel file exports to the C ABI layer (api.cu).
#pragma once

#include "common.cuh"

namespace lfgpu {

// assemble.cu
void launch_assembly(Context& c, int strategy);

// sparse.cu
void launch_find_diagonal(Context& c);
void launch_dirichlet(Context& c);           // elimination + zero-pivot sweep, in place on K, f
void launch_spmv_csr64(Context& c, const double* val, const double* x, double* y, const double* sub);
void launch_spmv_csr32(Context& c, const float* val, const float* x, float* y);
void launch_spmv_bsr64(Context& c, const double* x, double* y);
void launch_spmv_bsr32(Context& c, const float* x, float* y);
void ensure_bsr(Context& c);                 // BSR structure + FP64 values of K (constrained)
void ensure_bsr32(Context& c);
void ensure_csr32(Context& c);
// Jacobi inverse diagonal and 2x2 nodal factors; raises LFGPU_ERR_NONFINITE_DIAG
// when ``precond`` is Jacobi and a diagonal entry is not finite.
void ensure_preconditioners(Context& c, int precond);
void launch_to_float(Context& c, const double* in, float* out, i64 count);
double device_norm2(Context& c, const double* v, i64 count);      // synchronous helper
void launch_axpby(Context& c, i64 count, double a, const double* x, double b, double* y);

// pcg.cu
struct SolveSetup {
    int storage;
    int precond;
    double tolerance;
    i64 max_iterations;
    int mixed;
    int restart;
    double inner_reduction;
    i64 max_refinements;
    const double* x0;  // FP64 warm start or nullptr (x0 = 0)
    const double* rhs; // right-hand side (device)
    double* x;         // FP64 solution (device)
    int unrolled;      // profiling: plain graph of this many iterations instead of the conditional loop
};
PcgResult run_pcg(Context& c, const SolveSetup& s, float* kernel_ms);

// cg_graph.cu: the same solver as a device-driven CUDA graph of per-phase kernels
PcgResult run_cg_graph(Context& c, const SolveSetup& s, float* kernel_ms);
// FP64 PCG with a preconditioner applied by its own kernels inside the graph: the
// IC(0) triangular sweeps or the subdomain block solves.  apply_ms is the device
// time of one standalone application times the applications made.
PcgResult run_pcg_separate(Context& c, const SolveSetup& s, float* kernel_ms, double* apply_ms);
// One FP64 application z = M^-1 r of the built preconditioner, on the stream.
void launch_precond_apply(Context& c, int precond, const double* r, double* z);

// subdomain.cu: subdomain block-Jacobi split (per mesh and setting) and factor
// (per K version)
void ensure_subdomains(Context& c);
// Each block's inverse in FP32 (a D x D square) for the mixed loop, per K version.
void ensure_subdomain_inverse(Context& c);

// ic0.cu: IC(0) factor of the constrained K on its own pattern (built per K version)
enum Ic0Slot {
    kIc0Scale = 0,     // max |K(r, r)| as double bits (atomicMax)
    kIc0Breakdowns,    // pivots replaced by the floor
    kIc0MaxLevel,      // longest dependency chain of the factor, in rows
    kIc0FactorChunk,   // row-chunk counters of the factorisation and of the two sweeps
    kIc0ForwardChunk,
    kIc0BackwardChunk,
    kIc0Slots = 8
};
void ensure_ic0(Context& c);
// Level schedules of the two IC(0) sweeps, per pattern version (host schedule,
// uploaded); sets c.sweep_window (0 when the ring cannot hold the schedule).
void ensure_ic0_schedule(Context& c);
// The factor in schedule order for the level sweeps, per K version: FP64, and the
// FP32 copy when fp32 is set.  Requires ensure_ic0 and ensure_ic0_schedule.
void ensure_ic0_sweep_values(Context& c, bool fp32);
// Whether the level-scheduled sweeps run for this handle (option, schedule fit and,
// for LFGPU_IC0_SWEEP_AUTO, the average level width; `required`: the mixed loop,
// which has no other FP32 sweeps); throws LFGPU_ERR_UNSUPPORTED when they are
// required but the schedule does not fit.
bool ic0_use_levels(Context& c, bool required);
// The same choice for a schedule already built (no side effects).
bool ic0_levels_chosen(const Context& c, bool required);

// The level-scheduled sweeps run as one cluster of kSweepCluster CTAs of
// kSweepThreads consumer threads and a producer warp; every CTA keeps a ring of
// the last sweep_window results in shared memory and kSweepStages stages of
// operands, each one CTA's piece of one level (copied in by TMA).
constexpr int kSweepCluster = 8;
constexpr int kSweepThreads = 128;
constexpr int kSweepStages = 8;
constexpr int kSweepRingBars = 4;  // mbarriers cycling over the levels whose results are in flight
constexpr int kSweepRingMax = 16384;

#ifdef __CUDACC__
#define LF_HD __host__ __device__
#else
#define LF_HD
#endif

LF_HD inline int sweep_round16(int bytes) { return (bytes + 15) & ~15; }

// Byte offsets of a stage's arrays and its size, for elements of `elem` bytes and
// pieces of at most maxp rows and maxe entries.  Arrays that do not start on a
// 16-byte boundary are copied from the boundary below their start (TMA copies
// whole 16-byte units), hence the slack.
struct SweepStageLayout {
    int desc, dep, val, inv, rhs, rr, bytes;
};
LF_HD inline SweepStageLayout sweep_stage_layout(int elem, int maxp, int maxe) {
    SweepStageLayout l;
    l.desc = 0;
    l.dep = l.desc + sweep_round16(maxp * 16);
    l.val = l.dep + sweep_round16((maxe + 8) * 4);
    l.inv = l.val + sweep_round16((maxe + 8) * elem);
    l.rhs = l.inv + sweep_round16((maxp + 8) * elem);
    l.rr = l.rhs + sweep_round16((maxp + 8) * elem);
    l.bytes = l.rr + sweep_round16((maxp + 8) * elem);
    return l;
}
// Dynamic shared memory of a level sweep: the ring of `window` results, then the stages.
LF_HD inline int sweep_smem_bytes(int elem, int window, int maxp, int maxe) {
    return sweep_round16(window * elem) + kSweepStages * sweep_stage_layout(elem, maxp, maxe).bytes;
}
// Shared memory a sweep CTA may use beyond its dynamic part (barriers, pieces, reductions).
constexpr int kSweepStaticSmem = 4096;
// Elements allocated past the end of every array a sweep copies by TMA: a copy
// rounded up to whole 16-byte units reads up to three elements beyond its range.
constexpr int kSweepSlack = 16;

// pattern.cu: CSR pattern and element->value map on the device; false if a node
// has more elements than the device build handles (the caller builds on the host)
bool build_pattern_device(Context& c, std::vector<int>& rowptr_host);
// node -> elements lists in ascending element order, cached per mesh (c.ne_ptr, c.ne_list)
void ensure_node_elements(Context& c);
// Reverse Cuthill-McKee order of the mesh's node indices; false if a level is wider
// than the device search takes (the caller orders on the host)
bool rcm_device(Context& c, std::vector<int>& order);
// csr_profile of the pattern the mesh produces: nonzeros, bandwidth, profile; false
// if a node has more elements than the device build handles
bool mesh_profile_device(Context& c, long long out[3]);

// postprocess.cu: element fields (35 per element) and smoothed nodal stress (4 per node)
void launch_postprocess(Context& c, const double* u, double* fields, double* nodal);

// adjoint.cu
void launch_adjoint_grad(Context& c, const double* u, const double* lam, double* grad);

}  // namespace lfgpu
