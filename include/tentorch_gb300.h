/*
 * tentorch_gb300: the C ABI of the GB300 block-sparse contraction engine.
 *
 * A drop-in for the block-sparse contraction path of Jumqyc/TenTorch (`tensors.einsum` /
 * `contract` / `Tensor.place`).  The reference binds that path to Python with pybind11
 * (tentorch/_ext/bindings.cpp:250-361); this library exposes the same operations as plain C entry
 * points over integer handles and raw device pointers, so any host language binds it through its
 * FFI (the Python package `tentorch_gb300` binds it with ctypes).
 *
 * Model.  A category, a leg and a space (the shape of a tensor: category, codomain legs, domain
 * legs, total charge) are interned and named by int32 handles.  A tensor is a space plus one arena
 * of device memory holding every block, row major, at the offsets `tt_space_blocks` reports.  A
 * plan (a place, a contraction or an einsum) is compiled once per combination of spaces and cached;
 * executing it reads the operand arenas and writes the output arena on a CUDA stream, using a
 * caller-provided workspace.  The library never allocates arena memory.
 *
 * Conventions.  Sectors are passed as one int64 label (every category here has rank 1).  dtype 0 is
 * float64, 1 is complex128.  Every function returns a status: 0 on success, else one of TT_E*; the
 * message of the last failure on the calling thread is `tt_last_error()`.  Nothing throws across
 * the ABI.  Host-side functions (everything but tt_plan_execute / tt_plan_prepare / tt_dots) need no
 * GPU.
 */
#ifndef TENTORCH_GB300_H
#define TENTORCH_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TT_OK 0
#define TT_EINVAL 1 /* malformed request: the reference raises ValueError (std::invalid_argument) */
#define TT_ERANGE 2 /* lookup outside a tensor: IndexError (std::out_of_range) */
#define TT_ELOGIC 3 /* broken invariant: RuntimeError (std::logic_error / TORCH_CHECK) */
#define TT_ECUDA 4  /* a CUDA call failed: RuntimeError */

#define TT_DTYPE_FLOAT64 0
#define TT_DTYPE_COMPLEX128 1

#define TT_PRECISION_PER_BLOCK (-1) /* tt_plan_execute: one cuBLAS call per block pair */

typedef struct tt_plan tt_plan;

/* The message of the last failure on this thread. */
const char *tt_last_error(void);
/* The ABI version (monotone). */
int32_t tt_version(void);

/* ---- categories (tentorch/symmetry/cat/cat.h:190-429) ------------------------------------ */

/* kind: 0 no symmetry, 1 U(1), 2 SU(2), 3 Fibonacci, 4 Z_N (param = N), 5 fermion parity.
 * Replaces the module singletons of tentorch/_ext/bindings.cpp:464-470. */
int32_t tt_category(int32_t kind, int64_t param, int32_t *out);
/* Fusion outcomes of a x b in the category's order (FusionCategory::outcomes, cat.h:231).
 * Writes up to `cap` (sector, multiplicity) pairs, *n the total. */
int32_t tt_outcomes(int32_t cat, int64_t a, int64_t b, int32_t cap, int64_t *sectors, int32_t *mult, int32_t *n);
int32_t tt_dual(int32_t cat, int64_t a, int64_t *out);
int32_t tt_q_dim(int32_t cat, int64_t a, double *out);
/* F^d_{abc} (cat.h:282) / R_{bc} (cat.h:300) as row-major complex (re, im interleaved). */
int32_t tt_F_symbol(int32_t cat, int64_t a, int64_t b, int64_t c, int64_t d, int32_t cap, double *values,
                    int32_t *rows, int32_t *cols);
int32_t tt_R_symbol(int32_t cat, int64_t b, int64_t c, int32_t cap, double *values, int32_t *rows, int32_t *cols);

/* ---- legs and trees (tentorch/symmetry/tree/tree.h:33-199) ---------------------------------- */

/* Intern a leg (Leg::Leg, tree.cpp:90-140): blocks sorted by sector, distinct, positive. */
int32_t tt_leg(int32_t cat, int32_t n, const int64_t *sectors, const int64_t *mult, int32_t *out);
/* The blocks of a leg, sorted. */
int32_t tt_leg_blocks(int32_t leg, int32_t cap, int64_t *sectors, int64_t *mult, int32_t *n);
/* reachable_charges (tree.cpp:375-398). */
int32_t tt_reachable_charges(int32_t cat, int32_t nlegs, const int32_t *legs, int32_t cap, int64_t *out, int32_t *n);
/* fusion_trees (tree.cpp:400-471) flattened: per tree `nlegs` sectors, max(nlegs-2,0) inner
 * sectors, max(nlegs-1,0) copies, then the coupled sector; `stride` the int64 count per tree. */
int32_t tt_fusion_trees(int32_t cat, int32_t nlegs, const int32_t *legs, int64_t coupled, int64_t cap, int64_t *out,
                        int64_t *n_trees, int32_t *stride);

/* ---- spaces (tentorch/tensors/tensor.h:43-216, layout.h:64-127) --------------------------- */

/* Intern the shape of a tensor; its blocks follow block_keys (layout.cpp:34-47) in key order. */
int32_t tt_space(int32_t cat, int32_t ncod, const int32_t *cod, int32_t ndom, const int32_t *dom, int64_t qtotal,
                 int32_t *out);
/* Number of blocks and arena elements (block starts are 16-byte aligned, padding stays zero). */
int32_t tt_space_size(int32_t space, int64_t *nblocks, int64_t *elements);
/* Per block: (codomain root, domain root, copy) and (rows, cols, offset). */
int32_t tt_space_blocks(int32_t space, int64_t cap, int64_t *keys, int64_t *shapes);
/* The legs and charge of a space. */
int32_t tt_space_legs(int32_t space, int32_t cap, int32_t *legs, int32_t *ncod, int32_t *ndom, int64_t *qtotal);

/* ---- plans -------------------------------------------------------------------------------- */

/* Tensor::place(above, below) (tensors/place.cpp:183-247). */
int32_t tt_plan_place(int32_t space, int32_t nabove, const int32_t *above, int32_t nbelow, const int32_t *below,
                      tt_plan **out);
/* contract(left, right, left_legs, right_legs[, charge]) (linalg/graded/contract.cpp:117-175). */
/* The conjugate-transpose (bra) of a tensor of `space`: block (r, s, c) becomes block (s, r, c) of the
 * space with codomain and domain swapped and the dual charge, transposed and conjugated
 * (tentorch/tensors/tensor.cpp:99-107); one tiles pass. */
int32_t tt_plan_conj(int32_t space, tt_plan **out);
int32_t tt_plan_contract(int32_t left, int32_t right, int32_t n, const int32_t *left_legs, const int32_t *right_legs,
                         int32_t has_charge, int64_t charge, tt_plan **out);
/* einsum(spec, *operands, outcharge=) (linalg/graded/einsum.cpp:444-605, bindings.cpp:347-361). */
int32_t tt_plan_einsum(const char *spec, int32_t n, const int32_t *spaces, int32_t has_charge, int64_t charge,
                       tt_plan **out);
/* Drop every cached plan and its device tables (plans are cached per shape and live until this
 * call): every tt_plan pointer handed out before is invalid afterwards.  Synchronises the device
 * while it frees the tables. */
int32_t tt_plan_cache_clear(void);
/* The output space, workspace elements, GEMM flops, recoupled elements and op count of a plan. */
int32_t tt_plan_info(const tt_plan *plan, int32_t *out_space, int64_t *workspace, double *gemm_flops,
                     int64_t *moved_elements, int32_t *n_ops);
/* A text listing of the plan's operations and GEMM block shapes (m, n, K per pair), and for an
 * einsum the order it folds its operands in (einsum.cpp:216-301), for diagnosis; writes at most
 * cap-1 characters and a terminating zero, *length the full size. */
int32_t tt_plan_describe(const tt_plan *plan, int64_t cap, char *text, int64_t *length);
/* The gather index of operation `op` when it is a gather or a tiles pass (a composed chain of leg
 * moves whose F and R symbols are all 1; tiles are expanded entry by entry): output entry i reads
 * input entry index[i], -1 writes zero.  *count is the number of entries; nothing is written when
 * cap < *count.  For checking compiled leg moves against
 * the reference's per-step plans (tentorch/tensors/place.cpp:199-247). */
int32_t tt_plan_gather(const tt_plan *plan, int32_t op, int64_t cap, int32_t *index, int64_t *count);
/* Elements (float64-sized, or of the dtype if larger) of operand `i`'s prepared arena, 0 when the
 * operand needs no preparation.  The arena holds the operand after its leg moves and, for block
 * products that read it, its split-precision slices (cut once by tt_plan_prepare, read by every
 * split execution that is given the arena). */
int32_t tt_plan_prepared_size(const tt_plan *plan, int32_t operand, int64_t *elements);
/* Execute on `stream` (a cudaStream_t, 0 for the legacy stream).  precision 0: FP64 block
 * products in the grouped persistent kernels (a product whose result a leg move with unit
 * coefficients relabels for a second product, as in the two-site matvec, runs with that move and
 * that product as ONE launch; in split precision the first product stores through the move); k >= 1: split products on the tensor cores with k
 * bf16 slices per operand; TT_PRECISION_PER_BLOCK (-1): the plain per-block FP64 form, one cuBLAS
 * call per block pair as the reference issues them on a CUDA device
 * (tentorch/linalg/graded/contract.cpp:148-163), the comparison arm of the grouped kernels.
 * `prepared` (may be NULL, or hold NULLs) gives operands' prepared arenas from tt_plan_prepare.
 * `workspace` (tt_plan_info's elements of the dtype) must start zeroed: a plan with block products
 * keeps the counters of its split output tiles in the first 64 KiB, and every execution leaves
 * them zero again, so one zeroed workspace serves any number of executions of any plans on one
 * stream (they must not run concurrently on it). */
int32_t tt_plan_execute(const tt_plan *plan, int32_t dtype, int32_t precision, const void *const *inputs,
                        const void *const *prepared, void *output, void *workspace, void *stream);
/* `count` plans executed on `stream`, each as tt_plan_execute would (per plan its operand arenas
 * inputs[i], prepared arenas prepared[i] (may be NULL), output arena outputs[i] and its OWN workspace
 * workspaces[i], zeroed when first used).  When every plan is an FP64 product chain (the two-site
 * matvec: its operations besides the chain prepare operands) and count <= 64, the chains of all of
 * them run as ONE persistent launch, their work items dealt together over the SMs (the deal cached
 * per list of plans); otherwise, and in split precision, one plan after another.  *launched (may be
 * NULL) receives the number of launches of the plans' products made (1 for the batched one).  For
 * many independent DMRG windows of different bond dimension (tentorch/algorithms/dmrg.py:116-118 runs
 * one window at a time). */
int32_t tt_plan_execute_batch(int32_t count, const tt_plan *const *plans, int32_t dtype, int32_t precision,
                              const void *const *const *inputs, const void *const *const *prepared,
                              void *const *outputs, void *const *workspaces, void *stream, int32_t *launched);
/* The same as tt_plan_execute, synchronously, recording a CUDA event pair around every operation on
 * `stream`: per op its device milliseconds (-1 when it did not run) and its kind (0 zero, 1 gather,
 * 2 runs, 3 gemm, 4 add, 5 copy, 6 tiles, 7 a product, the leg move of its result and the product
 * that reads it run as one FP64 launch, timed on the first product's op).  For measurement; the
 * caller's stream is synchronised before it returns. */
int32_t tt_plan_execute_timed(const tt_plan *plan, int32_t dtype, int32_t precision, const void *const *inputs,
                              const void *const *prepared, void *output, void *workspace, void *stream, int32_t cap,
                              float *op_ms, int32_t *op_kind);
/* ---- autotuning: the forms of a plan's block products, chosen by timing, cached by histogram ---- */

/* The forms a plan's block products run in, as bits: TT_FORM_SEPARATE runs a product chain (two
 * products with the leg move between them, the two-site matvec) as separate launches instead of
 * one; TT_FORM_NO_TENSOR_CORES keeps split-precision products of large blocks on the mma.sync
 * kernel instead of the tcgen05 one.  Executions use the forms cached for the plan's block-size
 * histogram (0 when none is cached). */
#define TT_FORM_SEPARATE 1
#define TT_FORM_NO_TENSOR_CORES 2
/* The 64-bit key of the plan's block-size histogram: per block product the multiply-adds of its
 * block pairs binned by (log2 m, log2 n, log2 K), and whether it has a product chain. */
int32_t tt_plan_histogram(const tt_plan *plan, uint64_t *key);
/* Time every form that applies to the plan on these operands (arguments as tt_plan_execute; two
 * untimed and five timed executions of each on `stream`, synchronously), cache the fastest under
 * the plan's histogram for this dtype and precision, and return it (*forms) with its median time in
 * milliseconds (*ms).  Not capturable: a setup step, like the first execution of a plan. */
int32_t tt_autotune(const tt_plan *plan, int32_t dtype, int32_t precision, const void *const *inputs,
                    const void *const *prepared, void *output, void *workspace, void *stream, int32_t *forms, float *ms);
/* The forms cached for a histogram key, dtype and precision: *found 0 when there are none. */
int32_t tt_autotune_lookup(uint64_t key, int32_t dtype, int32_t precision, int32_t *forms, int32_t *found);
/* Cache forms for a key (a saved tuning table restored), or forget every cached choice. */
int32_t tt_autotune_store(uint64_t key, int32_t dtype, int32_t precision, int32_t forms);
int32_t tt_autotune_clear(void);

/* Run operand `operand`'s preparation only, writing its prepared arena (for float64 also the
 * slices of it that split-precision products read).  The arena stays valid while the operand's
 * arena is unchanged; a changed operand needs a new preparation. */
int32_t tt_plan_prepare(const tt_plan *plan, int32_t dtype, int32_t operand, const void *input, void *prepared,
                        void *workspace, void *stream);

/* ---- per-step plans, for checking against the reference (tensors/regroup.h:22-96) --------- */

/* The shifts of one step on one block of `space`: kind 0 exchange at `arm`, 1 bend down, 2 bend
 * up.  Per piece 8 doubles: first, last, from_step, to_step, run, re, im and the shift number;
 * per shift 9 int64 in `shifts`: from key (3), to key (3), rows, cols, piece count. */
int32_t tt_step_plan(int32_t space, int32_t kind, int32_t arm, int64_t key_cod, int64_t key_dom, int32_t key_copy,
                     int64_t cap_shifts, int64_t *shifts, int64_t cap_pieces, double *pieces, int64_t *n_shifts,
                     int64_t *n_pieces);
/* The chain of steps of a place: per step (kind, arm, space after). */
int32_t tt_chain(int32_t space, int32_t nabove, const int32_t *above, int32_t nbelow, const int32_t *below,
                 int32_t cap, int32_t *steps, int32_t *n);

/* ---- the Lanczos eigensolver of a window (tentorch/linalg/lanczos.py:8-64) ------------------ */

/* Doubles of scratch tt_lanczos needs for an arena of n entries and n_iter (1..60) steps. */
int32_t tt_lanczos_scratch(int64_t n, int32_t n_iter, int32_t dtype, int64_t *doubles);
/* The lowest eigenpair of the Hermitian action v -> plan(inputs with v as operand `vector_operand`)
 * by n_iter Krylov steps from `start` with full reorthogonalisation, all on `stream` with one host
 * synchronisation at the end (to read the energy and the size): *energy is the lowest Ritz value, `result` the normalised Ritz vector
 * and *size the Krylov dimension used (the steps before the first norm below `tol`, as the
 * reference stops).  The plan's output space must be the vector operand's space.  `prepared` as
 * for tt_plan_execute; `workspace` the plan's workspace; `scratch` tt_lanczos_scratch doubles. */
int32_t tt_lanczos(const tt_plan *plan, int32_t dtype, int32_t precision, const void *const *inputs,
                   const void *const *prepared, int32_t vector_operand, const void *start, int32_t n_iter,
                   double tol, void *workspace, void *scratch, void *result, double *energy, int32_t *size,
                   void *stream);
/* The same with no host wait at all (the tridiagonal's eigenpair is solved on the device): `energy`
 * and `size` are DEVICE pointers written on `stream`, like `result`.  The reference reads a norm and
 * inner products with .item() at every step (tentorch/linalg/lanczos.py:36-64,
 * tentorch/linalg/graded/compare.cpp:41). */
int32_t tt_lanczos_async(const tt_plan *plan, int32_t dtype, int32_t precision, const void *const *inputs,
                         const void *const *prepared, int32_t vector_operand, const void *start, int32_t n_iter,
                         double tol, void *workspace, void *scratch, void *result, double *energy, int32_t *size,
                         void *stream);

/* ---- truncating splittings (tentorch/linalg/graded/svd.cpp:41-177) -------------------------- */

/* Thin SVDs of `count` float64 blocks in one launch (one-sided Jacobi, mixed precision: FP32 sweeps,
 * then FP64 re-orthonormalisation and FP64 sweeps to full accuracy; blocks of 32 columns or more
 * sorted by column norm and QR-factored first, the sweeps then working on R^T; a thread-block
 * cluster per block; replaces the per-block at::linalg_svd of svd.cpp:57-62).  `table` is a DEVICE array of 7
 * int64 per block: a_off, rows, cols, u_off, s_off, vh_off, ws_off (offsets in doubles), best
 * ordered largest block first; `largest` is the largest min(rows, cols) among them (it sets the
 * cluster size).  Block i is rows x cols row-major at a + a_off; with k = min(rows, cols) <= 1024
 * it writes U (rows x k, row-major) at u + u_off, the k singular values in descending order at
 * s + s_off and Vh (k x cols, row-major) at vh + vh_off.  ws_off places the block's working set in
 * `workspace` (from tt_svd_workspace).  info[i] (device int32) receives the FP64 sweeps block i
 * took, -1 when they did not converge (then its factors are not to be used).  Asynchronous on
 * `stream`. */
int32_t tt_svd_blocks(int32_t count, int64_t largest, const int64_t *table, const double *a, double *u, double *s,
                      double *vh, double *workspace, int32_t *info, void *stream);
/* The workspace of tt_svd_blocks: for `count` blocks (host array of rows, cols per block) the
 * offset in doubles of each block's working set in the workspace (-1 for an empty block) and the
 * doubles the workspace needs in all. */
int32_t tt_svd_workspace(int32_t count, const int64_t *shapes, int64_t *offsets, int64_t *total);
/* Rank a split's singular values on the device (tentorch/linalg/graded/svd.cpp:68-118): `values`
 * (device, n_values) block after block, each block's `block_k[b]` values in descending order;
 * block b's domain sector id `block_sector[b]` and each sector's dual `dual[s]` (ids below
 * n_sectors; device int32 arrays).  The values above `tol` in descending order (ties by position),
 * at most `max_bond` of them (-1: no cap), then the +-q pairing of the bond: kept[b] (device int32)
 * receives how many leading values block b keeps.  One CTA; TT_EINVAL when the values do not fit
 * its shared memory (about 16K values), nothing launched. */
int32_t tt_svd_rank(const double *values, int32_t n_values, const int32_t *block_k, const int32_t *block_sector,
                    int32_t n_blocks, const int32_t *dual, int32_t n_sectors, double tol, int64_t max_bond, int32_t *kept,
                    void *stream);
/* Write the kept part of the factors of tt_svd_blocks into the two tensors of a split, one CTA per
 * kept block.  `table` is a DEVICE array of 10 int64 per block: u_off, s_off, vh_off (packed
 * factors), first_off, second_off (the blocks of the two output arenas), values_off (the kept
 * values' place in the bond array), then rows, cols, k, kept, first_ld, column, row, absorb as
 * int32 pairs packed into 4 int64 (rows | cols << 32, k | kept << 32, first_ld | column << 32,
 * row | absorb << 32).  first[:, column:column+kept] = U[:, :kept], second[row:row+kept, :] =
 * Vh[:kept, :], values = s[:kept], with the values multiplied into U (absorb 1), Vh (2) or their
 * square roots into both (3). */
int32_t tt_svd_keep(int32_t count, const int64_t *table, const double *u, const double *s, const double *vh,
                    double *first, double *second, double *values, void *stream);

/* ---- Krylov arithmetic on arenas ----------------------------------------------------------- */

/* out[2j], out[2j+1] = <a_j, b> (conjugating a_j) for j < count, on `stream`, with no host
 * synchronisation; `as` is a device array of `count` arena pointers, n the arena elements,
 * `scratch` 2*120*count doubles of device memory. */
int32_t tt_dots(int32_t dtype, int32_t count, const void *const *as, const void *b, int64_t n, double *scratch,
                double *out, void *stream);

/* tt_dots without caller scratch, for callers that cannot allocate device memory where they need
 * the dot products (a host framework that forbids allocation inside its solver loop, or one whose
 * memory pool belongs to another runtime).  It has no counterpart in the reference.  The partial
 * sums live in a static device array of this library (120 KiB on every GPU that loads it, held
 * until the process exits), so `count` is at most 64 (TT_EINVAL beyond).  The first call on a
 * device looks up that array's device address (make it before any stream capture); calls whose
 * work overlaps on the GPU share the array and race.  Otherwise the same contract as tt_dots. */
int32_t tt_dots_noalloc(int32_t dtype, int32_t count, const void *const *as, const void *b, int64_t n, double *out,
                        void *stream);
/* Copy `bytes` between page-locked host memory and device memory with a kernel that reads or
 * writes the host end directly over the coherent CPU-GPU link (GB300's NVLink-C2C), on `stream`:
 * direction 0 host -> device (src host, dst device), 1 device -> host.  The host end must be
 * mapped page-locked memory (cudaHostAlloc; TT_EINVAL otherwise, nothing copied).  The transfer a
 * step of the end-to-end matvec makes (its vector in, its image out) without a copy-engine call.
 * No counterpart in the reference (its tensors live on one device). */
int32_t tt_link_copy(void *dst, const void *src, int64_t bytes, int32_t direction, void *stream);

#ifdef __cplusplus
}
#endif

#endif
