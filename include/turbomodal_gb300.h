/*
 * turbomodal_gb300 C ABI: GB300 (sm_103a) cyclic-symmetry modal solve.
 *
 * Plain C: opaque context, POD descriptors, caller-owned output buffers, int status
 * codes (TMG_OK == 0) and a per-context last-error string.  No exception crosses the ABI.
 * A context drives one CUDA device; its calls are not thread-safe with each other
 * (one host thread per context).
 *
 * Each entry point names the reference interface it replaces (file:line in the
 * turbomodal project).
 */
#ifndef TURBOMODAL_GB300_H
#define TURBOMODAL_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TMG_OK 0
#define TMG_ERR_ARG 1      /* invalid argument / size */
#define TMG_ERR_CUDA 2     /* CUDA runtime error (message in tmg_last_error) */
#define TMG_ERR_STATE 3    /* call out of order (e.g. no sector uploaded) */
#define TMG_ERR_NUMERIC 4  /* zero pivot, singular Jacobian, breakdown */
#define TMG_ERR_NOMEM 5    /* device memory budget exceeded */
#define TMG_ERR_TIMEOUT 6  /* a bounded device wait gave up */

/* Matrix selectors for tmg_assemble / tmg_projection. */
#define TMG_MAT_K 0        /* sector stiffness            assembler.cpp:11-69   */
#define TMG_MAT_M 1        /* sector consistent mass      assembler.cpp:11-69   */
#define TMG_MAT_KOMEGA 2   /* spin softening at rpm       assembler.cpp:157-218 */
#define TMG_MAT_G 3        /* gyroscopic (no 2*omega)     assembler.cpp:157-218 */
#define TMG_MAT_KSIGMA 4   /* stress stiffening at rpm    assembler.cpp:71-155  */
#define TMG_MAT_KEFF 5     /* K - Komega + Ksigma         cyclic_solver.cpp:744-773 */
#define TMG_MAT_KCF 10     /* free-space projections      cyclic_solver.cpp:560-671 */
#define TMG_MAT_KPF 11
#define TMG_MAT_MCF 12
#define TMG_MAT_MPF 13
#define TMG_MAT_GCF 14
#define TMG_MAT_GPF 15
#define TMG_MAT_K0R 20     /* real k=0 / k=N/2 matrices   cyclic_solver.cpp:673-723 */
#define TMG_MAT_M0R 21
#define TMG_MAT_KHR 22
#define TMG_MAT_MHR 23
#define TMG_MAT_KK 30      /* per-harmonic K_k, M_k       cyclic_solver.cpp:942-947 */
#define TMG_MAT_MK 31
#define TMG_MAT_L1 32      /* Lancaster L1 = [[i 2 omega G_k, K_k], [K_k, 0]]  modal_solver.cpp:151-177 */
#define TMG_MAT_L2 33      /* Lancaster L2 = [[M_k, 0], [0, K_k]]             modal_solver.cpp:179-198 */

/* Arithmetic of the shift-invert factorisation and triangular solves. */
#define TMG_PREC_FP64 0    /* plain FP64 supernodal LDL^H */
#define TMG_PREC_MIXED 1   /* FP32 LDL^H + FP64 iterative refinement of every solve */

typedef struct tmg_context tmg_context;

/* Sector mesh + material + cyclic boundary data.
 * Replaces the state the reference CyclicSymmetrySolver constructor captures
 * (cyclic_solver.cpp:88-105, mesh.hpp:40-53, material.cpp:5-13). */
typedef struct {
    int32_t num_nodes;
    const double* coords;            /* num_nodes x 3, row-major */
    int32_t num_elements;
    const int32_t* connectivity;     /* num_elements x 10, TET10 node order of element.cpp:71-85 */
    double E, nu, rho;
    int32_t num_sectors;
    int32_t rotation_axis;           /* 0 = X, 1 = Y, 2 = Z */
    int32_t num_left;
    const int32_t* left_nodes;       /* matched left boundary nodes  */
    int32_t num_right;
    const int32_t* right_nodes;      /* matched right boundary nodes */
    int32_t num_pairs;
    const int32_t* pairs;            /* (left, right) x num_pairs    */
    int32_t num_constrained;
    const int32_t* constrained_nodes;/* FIXED hub nodes (empty = free hub) */
} tmg_sector_desc;

/* Per-result metadata of a ModalResult (modal_solver.hpp:8-15). */
typedef struct {
    int32_t harmonic_index;
    int32_t num_modes;
    int32_t converged;
    int32_t iterations;              /* Lanczos restarts used */
    int32_t status;                  /* TMG_OK or the per-problem error code */
    double rpm;
    double max_residual;             /* max ||K x - lambda M x|| / ||K x|| over modes */
    double refine_residual;          /* worst relative residual of a refined solve (mixed) */
} tmg_result_meta;

/* Context on one device with a device-memory budget (0 = 90% of free memory).
 * Replaces the per-solver thread pool + memory cap (cyclic_solver.cpp:1226-1273). */
int tmg_create(int device, size_t mem_budget_bytes, tmg_context** out);

/* Change the device-memory budget of later solves (0 = 90% of the memory free now); the
 * number of problems factorised together is chosen to fit it.  Replaces the
 * memory_reserve_fraction argument of solve_at_rpm (python_bindings.cpp:340-360,
 * cyclic_solver.cpp:1226-1273). */
int tmg_set_memory_budget(tmg_context* ctx, size_t mem_budget_bytes);

/* Options of later solves (tmg_set_option / tmg_get_option).
 * TMG_OPT_SHIFT: the shift sigma of the standard path's shift-invert operator K_k - sigma M_k
 *   (default 1.0, the value the reference hardcodes at cyclic_solver.cpp:1017).  An extension
 *   of the reference, which has no such argument.
 * TMG_OPT_DEFLATE: 1 = deflate the FP64 refinement CG of a mixed solve with the lowest
 *   eigenvectors each complex harmonic found at the previous speed of the same operator
 *   pattern (default 0).  Method change only: results equal the undeflated ones to the
 *   refinement tolerance.
 * TMG_OPT_TENSOR_CORES: 1 = the complex FP32 factorisation of the mixed path runs its large
 *   trailing Schur updates on the tensor cores (tcgen05, three-way BF16 split with FP32
 *   accumulation); 0 = on the FP32 SIMT pipe (default 0: on the config-1 sector the tensor-core
 *   factor took as long and its refined solves needed about a quarter more FP32 solves).
 *   Method change only, as above.
 * TMG_OPT_AUTOTUNE: 1 = the first solve on a new complex operator pattern times candidate
 *   supernode shapes (relaxed amalgamation, front width cap, tensor-core row threshold) on its
 *   own operator values and keeps the fastest, cached per pattern for the process (default 0).
 *   tmg_tuning_report lists the trials.
 * TMG_OPT_REFINE_TOL: relative residual ||b - A x|| / ||b|| at which the FP64 refinement of a
 *   mixed-precision shift-invert solve stops (default 1e-10, accepted range [1e-14, 1e-6]); a
 *   problem whose refinement stalls above 100x the target is solved again in FP64. */
#define TMG_OPT_SHIFT 0
#define TMG_OPT_DEFLATE 1
#define TMG_OPT_TENSOR_CORES 2
#define TMG_OPT_AUTOTUNE 3
#define TMG_OPT_REFINE_TOL 4
int tmg_set_option(tmg_context* ctx, int option, double value);
int tmg_get_option(tmg_context* ctx, int option, double* value);
int tmg_destroy(tmg_context* ctx);
const char* tmg_last_error(const tmg_context* ctx);

/* Upload a sector; replaces CyclicSymmetrySolver(mesh, material, fluid, apply_hub)
 * (python_bindings.cpp:321-331, cyclic_solver.cpp:88-105). */
int tmg_upload_sector(tmg_context* ctx, const tmg_sector_desc* desc);

/* Assemble one sector matrix on the device and copy it out as CSC (column pointers,
 * sorted row indices, FP64 values).  Pass NULL arrays to query *nnz first.
 * Replaces GlobalAssembler::assemble / K() / M() / K_omega() / G() / K_sigma()
 * (assembler.cpp:11-218, python_bindings.cpp:162-197). */
int tmg_assemble(tmg_context* ctx, int which, double rpm, int64_t* nnz,
                 int32_t* colptr, int32_t* rowidx, double* values);

/* Build the rotating-effect operators and the cyclic projections at one speed
 * (cyclic_solver.cpp:735-899). */
int tmg_prepare(tmg_context* ctx, double rpm, int coriolis);

/* Copy a projected matrix (complex interleaved values) after tmg_prepare.
 * k selects the harmonic for TMG_MAT_KK / TMG_MAT_MK, which are returned on the union of the
 * projections' structural patterns (the operator the solver factorises): entries that the
 * reference's pruning removes as roundoff are present as exact zeros.  TMG_MAT_L1 / TMG_MAT_L2
 * (after tmg_prepare with coriolis at a nonzero speed, 0 < k <= N/2) are the 2n x 2n matrices of
 * the Coriolis QEP, both on the pattern of the shifted operator L1 - sigma L2 (*n = 2n).  Pass
 * NULL arrays to query. */
int tmg_projection(tmg_context* ctx, int which, int k, int64_t* nnz, int32_t* n,
                   int32_t* colptr, int32_t* rowidx, double* values);

/* Fill-reducing order, elimination tree and L column counts of the shift-invert operator
 * K_k - sigma M_k (kind 0: complex harmonics; 1: k = 0; 2: k = N/2), as the reference's
 * SimplicialLDLT<..., Lower>::analyzePattern computes them (hermitian_lanczos.cpp:20).
 * perm[j] = original index of pivot j.  Pass NULL arrays to query *n. */
int tmg_symbolic(tmg_context* ctx, int kind, int32_t* n, int32_t* perm, int32_t* parent,
                 int32_t* colcount);

/* Size of the symbolic factorisation of kind (see tmg_symbolic; 3: the Coriolis QEP operator
 * L1 - sigma L2 after tmg_prepare with coriolis), 10 doubles: out[0] n, [1] nnz(L)
 * of the simplicial factor, [2] supernodes, [3] tree levels, [4] largest front, [5] L-panel
 * storage entries per problem, [6] factorisation flops (real; complex arithmetic counted x4),
 * [7] operator lower-triangle entries, [8] update-block workspace entries per problem,
 * [9] L entries read by one triangular solve. */
int tmg_symbolic_stats(tmg_context* ctx, int kind, double* out);

/* Full modal solve at one speed; replaces CyclicSymmetrySolver::solve_at_rpm
 * (cyclic_solver.cpp:725-1357, python_bindings.cpp:332-361).  harmonics == NULL or
 * nh == 0 solves k = 0..N/2.  Results stay in the context until the next solve. */
int tmg_solve_at_rpm(tmg_context* ctx, double rpm, int num_modes, const int32_t* harmonics, int nh,
                     int coriolis, double min_frequency, int precision, int32_t* num_results);

/* Modal solves at several speeds; replaces CyclicSymmetrySolver::solve_rpm_sweep
 * (cyclic_solver.cpp:1359-1373), which calls solve_at_rpm once per speed.  On the standard path
 * the harmonics of several speeds (consecutive speeds with the same operator pattern, as many
 * as the memory budget holds) are factorised and iterated as one batch; each result equals
 * what tmg_solve_at_rpm returns at its speed.  Results: speed-major in the order of rpms,
 * harmonics ascending within a speed (tmg_result_info gives each one's rpm and k); a failed
 * harmonic keeps its place with a nonzero status. */
int tmg_solve_sweep(tmg_context* ctx, const double* rpms, int nrpm, int num_modes, const int32_t* harmonics, int nh,
                    int coriolis, double min_frequency, int precision, int32_t* num_results);

/* Result access (ModalResult fields, modal_solver.hpp:8-15).  shapes: num_dof x num_modes
 * complex interleaved, column-major; NULL skips the copy. */
int tmg_result_info(tmg_context* ctx, int idx, tmg_result_meta* info);
int tmg_result_copy(tmg_context* ctx, int idx, double* freqs, double* shapes, int32_t* whirl);

/* Device memory this context holds now (*current: sector data, operators, symbolic
 * analyses, results of the last solve kept for copying) and the most it held since creation or
 * tmg_reset_peak_bytes (*peak), in bytes; either pointer may be NULL.  For admission control
 * of concurrent contexts; no counterpart in the reference, which runs on the CPU. */
int tmg_device_bytes(tmg_context* ctx, int64_t* current, int64_t* peak);
int tmg_reset_peak_bytes(tmg_context* ctx);

/* Trials of the last supernode-shape tuning (TMG_OPT_AUTOTUNE); no counterpart in the reference,
 * whose simplicial factorisation has no tile shapes.  *rows = number of trials; out (may be NULL)
 * receives min(max_rows, *rows) rows of 9 doubles: relax, front width cap, tensor-core row
 * threshold, factorisation ms, ms per batched triangular solve, score ms, L entries per problem,
 * supernodes, chosen (1/0). */
int tmg_tuning_report(tmg_context* ctx, double* out, int max_rows, int* rows);

/* Modal mass of every mode of a result, N * Re(phi^H M_sector phi) in kg over the full annulus,
 * computed on the device from the expanded shapes and the sector mass matrix.  Replaces the
 * reference's _modal_mass_from_M over a second host assembly (python/turbomodal/solver.py:91-114).
 * mass: num_modes doubles. */
int tmg_result_modal_mass(tmg_context* ctx, int idx, double* mass);

/* Time (ms) of the phases of the last tmg_solve_at_rpm: [0] prepare (assembly, prestress,
 * projections), [1] factorisations, [2] Lanczos, [3] post-processing, [4] the whole call
 * measured with CUDA events on the context's stream; counts: [5] batched triangular solves,
 * [6] shift-invert applications, [7] most refinement iterations of one application, [8] problems
 * of a mixed-precision batch solved again on the FP64 path (an FP32 zero pivot, a breakdown or
 * a refinement that stalled; cyclic_solver.cpp:1334-1342 retries failed harmonics likewise); and
 * the number of this library's kernel launches in it. */
int tmg_last_timing(tmg_context* ctx, double* phase_ms, int nphase, int64_t* kernel_launches);

/* Profiling mode (measurement only; it synchronises after every triangular solve): CUDA-event
 * time of each shift-invert triangular-solve graph.  tmg_profile_solve returns out[0] number of
 * solves, out[1] total ms, out[2] algorithmic bytes (stored L entries read once per sweep
 * direction + the solution vector), accumulated since tmg_set_profiling. */
int tmg_set_profiling(tmg_context* ctx, int on);
int tmg_profile_solve(tmg_context* ctx, double* out);

/* Complex FP64 entries the static scratch of tmg_projection_harmonic_static holds (8 MiB). */
#define TMG_STATIC_SCRATCH_ENTRIES 524288

/* tmg_projection for TMG_MAT_KK / TMG_MAT_MK with no device allocation: no counterpart in the
 * reference (its per-harmonic sums, cyclic_solver.cpp:942-947, run on the CPU).  The matrix is
 * formed in one file-scope __device__ array of TMG_STATIC_SCRATCH_ENTRIES complex entries per
 * device instead of a per-call device buffer; the call makes no cudaMalloc / cudaFree and no
 * other allocating call, and its output equals tmg_projection's.  For callers that cannot
 * allocate device memory at that point: a process whose whole device budget is committed to
 * resident factors and Lanczos bases, or a host thread that must not wait on the device-wide
 * synchronisation cudaFree performs.
 *  - A matrix with more than TMG_STATIC_SCRATCH_ENTRIES entries is rejected with TMG_ERR_ARG
 *    (*nnz is still set); use tmg_projection for it.
 *  - No scratch entry needs to start at zero: every entry copied out is written first.
 *  - One scratch array per device is shared by every context on that device: calls that
 *    overlap in time on one device (two host threads, or two contexts) race on it.  The call
 *    synchronises its stream before returning, so calls made one after another are safe.
 *  - Every call made outside a stream capture looks the array's address up
 *    (cudaGetSymbolAddress, with the context's device current), so a primary context that was
 *    reset and re-created is followed; a call made during a capture reuses the address of the
 *    last call outside one.  Make the first call on a device before any stream capture begins.
 * Pass NULL arrays to query *nnz and *n. */
int tmg_projection_harmonic_static(tmg_context* ctx, int which, int k, int64_t* nnz, int32_t* n,
                                   int32_t* colptr, int32_t* rowidx, double* values);

#ifdef __cplusplus
}
#endif
#endif /* TURBOMODAL_GB300_H */
