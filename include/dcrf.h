/*
 * dcrf.h -- C ABI of the GB300 dense-CRF engine (libdcrf_gb300.so).
 *
 * Drop-in boundary for the mean-field path of pydensecrf: each entry point
 * names the reference interface it replaces (paths inside the pydensecrf
 * project).  The reference binds its C++ core through Cython
 * (pydensecrf/densecrf.pxd:47-84); this library exposes the same operations as
 * plain C with opaque handles, integer status codes and raw pointers.
 *
 * Conventions
 *   - Every function returns DCRF_OK (0) or a negative DCRF_ERR_* code; the
 *     message of the last failure on the calling thread is available from
 *     dcrf_last_error().  (The reference raises C++ exceptions that Cython
 *     maps to Python exceptions: densecrf.pxd:9-26.)
 *   - `where` says whether a pointer is host (DCRF_HOST) or device
 *     (DCRF_DEVICE) memory; host buffers are copied through the handle's
 *     stream, device buffers are used in place.
 *   - Label-major layout (DCRF_LAYOUT_LM): an M x N quantity is stored as M
 *     rows of N floats -- the numpy (M, N) C-order array that
 *     DenseCRF.setUnaryEnergy takes (densecrf.pyx:80-89).  Point-major
 *     (DCRF_LAYOUT_PM): N rows of M floats -- the memory of the reference's
 *     column-major Eigen MatrixXf that inference() returns (eigen.pyx:68-81).
 *   - Features are (d, N) C-order (densecrf.pyx:71-75).
 *   - A handle is used by one host thread at a time; all work of a handle is
 *     ordered on its stream.  Calls return after the result is complete (the
 *     host-visible outputs are written) unless stated otherwise.
 *   - Lattice arithmetic: the reference compiles a different lattice build on
 *     x86 (SSE) and on other hosts (scalar) (permutohedral.cpp:36-47,
 *     140-474).  DCRF_VARIANT_SSE (the default) reproduces the x86 build,
 *     DCRF_VARIANT_SCALAR the scalar build, table for table.
 */
#ifndef DCRF_GB300_H
#define DCRF_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DCRF_ABI_VERSION 1

/* status codes */
#define DCRF_OK 0
#define DCRF_ERR_INVALID_ARG -1  /* bad shape, null pointer, unsupported size */
#define DCRF_ERR_CUDA -2         /* a CUDA runtime call failed */
#define DCRF_ERR_OOM -3          /* device allocation failed */
#define DCRF_ERR_HASH_FULL -4    /* lattice hash table overflowed (internal retry failed) */
#define DCRF_ERR_KEY_OVERFLOW -5 /* a lattice coordinate left the int16 range of the reference's keys */
#define DCRF_ERR_NO_DEVICE -6    /* no usable CUDA device */
#define DCRF_ERR_STATE -7        /* call not valid in the handle's current state */
#define DCRF_ERR_TIMEOUT -8      /* a bounded device-side wait gave up */

#define DCRF_HOST 0
#define DCRF_DEVICE 1

#define DCRF_LAYOUT_LM 0 /* label-major: M rows of N */
#define DCRF_LAYOUT_PM 1 /* point-major: N rows of M */

#define DCRF_VARIANT_SSE 0
#define DCRF_VARIANT_SCALAR 1

/* enums of pydensecrf/densecrf/include/pairwise.h:32-42 (same values) */
#define DCRF_NO_NORMALIZATION 0
#define DCRF_NORMALIZE_BEFORE 1
#define DCRF_NORMALIZE_AFTER 2
#define DCRF_NORMALIZE_SYMMETRIC 3
#define DCRF_CONST_KERNEL 0
#define DCRF_DIAG_KERNEL 1
#define DCRF_FULL_KERNEL 2

/* label compatibility kinds (labelcompatibility.h:44-88) */
#define DCRF_COMPAT_POTTS 0    /* compat = &w (1 float):     out = -w * Q          */
#define DCRF_COMPAT_DIAGONAL 1 /* compat = v (M floats):      out = diag(v) Q       */
#define DCRF_COMPAT_MATRIX 2   /* compat = m (M*M, row-major): out = 1/2(m+m^T) Q   */

typedef struct dcrf_crf dcrf_crf;

/* ABI version (DCRF_ABI_VERSION). No reference counterpart. */
int dcrf_abi_version(void);

/* Copies the last error message of the calling thread into buf (always
 * NUL-terminated when len > 0); returns the last status code.  Replaces the
 * exception text the Cython layer raises (densecrf.pyx:73,82,134,136). */
int dcrf_last_error(char *buf, size_t len);

/* DenseCRF(N, M): densecrf.pyx:51-63 -> densecrf.cpp:39-40.
 * Binds the handle to the current CUDA device and creates its own stream.
 * M may be 1 .. DCRF_MAX_LABELS (4096).  With more than 32 labels the labels
 * are processed in chunks of 32: inference, start/step, klDivergence, map,
 * both debug energies, the logistic unary and the raw filters work as for any
 * M; the adjoint (dcrf_inference_checkpointed, dcrf_backward) returns
 * DCRF_ERR_INVALID_ARG. */
int dcrf_create(int N, int M, dcrf_crf **out);

/* DenseCRF2D(W, H, M): densecrf.pyx:107-118 -> densecrf.cpp:47-48. */
int dcrf_create_2d(int W, int H, int M, dcrf_crf **out);

/* Batches (no reference counterpart: the reference solves one DenseCRF per
 * object).  One handle holds n_images independent problems with the same M
 * and the same pairwise terms: N[b] points each (dcrf_create_batch, features
 * given by dcrf_add_pairwise) or W[b] x H[b] pixels each
 * (dcrf_create_batch_2d, dcrf_add_pairwise_gaussian/_bilateral with the
 * images' RGB bytes one after another).  Points are numbered image after
 * image.  Every image gets its own lattice (the image index is part of the
 * lattice key), so results per image are those of a separate handle; all
 * images run in the same launches.  Label-major buffers hold image b's
 * M x N[b] block after those of images < b; point-major buffers are
 * [sum N][M].  dcrf_kl_divergence sums over the images; compatibility and
 * kernel gradients of dcrf_backward are summed over the images (shared
 * parameters). */
int dcrf_create_batch(int n_images, const int *N, int M, dcrf_crf **out);
int dcrf_create_batch_2d(int n_images, const int *W, const int *H, int M, dcrf_crf **out);
/* Number of images and their point offsets (n_images + 1 ints; either may be NULL). */
int dcrf_batch_info(dcrf_crf *h, int *n_images, int *point_start);

/* Destructor: densecrf.pyx:65-69 -> densecrf.cpp:41-46. NULL is a no-op. */
int dcrf_destroy(dcrf_crf *h);

/* Orders the handle's work on a caller-provided cudaStream_t (NULL restores
 * the handle's own stream).  No reference counterpart (the reference is
 * synchronous CPU code). */
int dcrf_set_stream(dcrf_crf *h, void *cuda_stream);

/* Selects the lattice arithmetic (DCRF_VARIANT_*) for terms added after the
 * call; see the file comment.  No reference counterpart (compile-time there). */
int dcrf_set_variant(dcrf_crf *h, int variant);

/* setUnaryEnergy(u): densecrf.pyx:80-89 -> densecrf.cpp:89-91
 * (ConstUnaryEnergy, unary.cpp:42-46).  U is M x N in `layout`. */
int dcrf_set_unary(dcrf_crf *h, const float *U, int layout, int where);

/* setUnaryEnergy(L, f) / LogisticUnary(L, f): densecrf.pyx:44-46,80-89 ->
 * LogisticUnaryEnergy (unary.cpp:48-52): U = L f, computed on the device into
 * the unary rows.  L is M x nfeat and f is nfeat x N, both C-order in `where`.
 * Later dcrf_set_unary_parameters calls change L and recompute U. */
int dcrf_set_unary_logistic(dcrf_crf *h, const float *L, int nfeat, const float *f, int where);

/* addPairwiseEnergy(features, compat, kernel, normalization):
 * densecrf.pyx:71-75 -> densecrf.cpp:54-57 -> pairwise.cpp:116-122,170-172.
 * feat is (d, N) C-order.  Builds the lattice and the normalisation on the
 * device.  The compat buffer is copied (the reference takes ownership of a heap
 * object, densecrf.pyx:11-20).  *term_out (may be NULL) receives the term index. */
int dcrf_add_pairwise(dcrf_crf *h, const float *feat, int d, int where, int compat_kind, const float *compat,
                      int kernel_type, int normalization_type, int *term_out);

/* DenseCRF2D.addPairwiseGaussian(sxy, compat, kernel, normalization):
 * densecrf.pyx:120-124 -> densecrf.cpp:61-69; features (i/sx, j/sy) for pixel
 * j*W+i are generated on the device. */
int dcrf_add_pairwise_gaussian(dcrf_crf *h, float sx, float sy, int compat_kind, const float *compat,
                               int kernel_type, int normalization_type, int *term_out);

/* DenseCRF2D.addPairwiseBilateral(sxy, srgb, rgbim, compat, ...):
 * densecrf.pyx:126-140 -> densecrf.cpp:70-81. rgb is H x W x 3 uint8, C-order. */
int dcrf_add_pairwise_bilateral(dcrf_crf *h, float sx, float sy, float sr, float sg, float sb, const uint8_t *rgb,
                                int where, int compat_kind, const float *compat, int kernel_type,
                                int normalization_type, int *term_out);

/* inference(n): densecrf.pyx:91-92 -> densecrf.cpp:115-131.  Writes the M x N
 * marginals to Q in `layout`. */
int dcrf_inference(dcrf_crf *h, int n_iterations, float *Q, int layout, int where);

/* startInference(): densecrf.pyx:94-95 -> densecrf.cpp:178-186 (all zeros when
 * no unary is set). */
int dcrf_start_inference(dcrf_crf *h, float *Q, int layout, int where);

/* stepInference(Q, tmp1, tmp2): densecrf.pyx:97-98 -> densecrf.cpp:187-201.
 * One mean-field update of Q, in place. */
int dcrf_step_inference(dcrf_crf *h, float *Q, int layout, int where);

/* klDivergence(Q): densecrf.pyx:100-101 -> densecrf.cpp:214-235.  Accumulated
 * in double on the device (the reference sums the pairwise term in float). */
int dcrf_kl_divergence(dcrf_crf *h, const float *Q, int layout, int where, double *kl_out);

/* map(n): densecrf.cpp:132-137 + currentMap 202-211 (declared but not wrapped
 * by densecrf.pxd:61-62): argmax labels (first maximum) after n iterations. */
int dcrf_map(dcrf_crf *h, int n_iterations, int16_t *labels, int where);

/* DenseCRF::unaryEnergy (densecrf.cpp:141-153; C++ only, not wrapped by the
 * reference's Cython): energy[i] = U(l_i, i) for 0 <= l_i < M, else 0.  labels
 * are N int16 in `where`; energy is N floats in `where_out`. */
int dcrf_unary_energy(dcrf_crf *h, const int16_t *labels, int where, float *energy, int where_out);

/* DenseCRF::pairwiseEnergy (densecrf.cpp:154-177): energy[i] = -1/2 times the
 * message of term `term` (-1: the sum over all terms) at l_i for the one-hot
 * labelling, 0 where l_i is not a label. */
int dcrf_pairwise_energy(dcrf_crf *h, const int16_t *labels, int where, int term, float *energy, int where_out);

/* Blocks until the handle's stream is idle. */
int dcrf_synchronize(dcrf_crf *h);

/* Removes every pairwise term (frees their lattices); the unary stays.  No
 * reference counterpart (a reference user creates a new DenseCRF instead);
 * lets one handle solve a sequence of images without reallocating. */
int dcrf_clear_pairwise(dcrf_crf *h);

/* ---- learning: parameters and the adjoint --------------------------------- */

/* Replaces term `term`'s label compatibility (kind and values as in
 * dcrf_add_pairwise).  Counterpart of LabelCompatibility::setParameters /
 * DenseCRF::setLabelCompatibilityParameters (labelcompatibility.cpp:54-56,
 * 73-75,95-100; densecrf.cpp:321-333), with full values instead of the
 * reference's packed vector. */
int dcrf_set_compat(dcrf_crf *h, int term, int compat_kind, const float *compat);

/* Kernel parameters of term `term` (DenseKernel::setParameters,
 * pairwise.cpp:140-151): DIAG_KERNEL d scales p (features become p_j * f_j),
 * FULL_KERNEL a d x d matrix P, row-major (features become P f).  Rebuilds the
 * lattice and the normalisation.  CONST_KERNEL has no parameters. */
int dcrf_set_kernel_params(dcrf_crf *h, int term, const float *params);

/* The reference's parameter vectors (densecrf.cpp:298-360).  Each getter
 * writes the count to *n (may be NULL) and, when out is non-NULL, the values
 * (DCRF_ERR_INVALID_ARG if capacity < count); each setter takes exactly that
 * many values.
 *   unary: a logistic unary's L in column-major order, m + M j
 *          (LogisticUnaryEnergy::parameters, unary.cpp:53-57); none for a
 *          constant unary (unary.cpp:32-36).
 *   label compatibility: the terms' LabelCompatibility::parameters one after
 *          another -- Potts w; Diagonal the M weights; Matrix the upper
 *          triangle of the symmetric matrix row by row, M(M+1)/2 values
 *          (labelcompatibility.cpp:50-54,69-71,88-100).
 *   kernel: the terms' DenseKernel::parameters one after another -- DIAG the d
 *          feature scales, FULL the d x d matrix column-major, CONST none
 *          (pairwise.cpp:129-151); setting them rebuilds the lattices. */
int dcrf_unary_parameters(dcrf_crf *h, float *out, int capacity, int *n);
int dcrf_set_unary_parameters(dcrf_crf *h, const float *v, int n);
int dcrf_label_compatibility_parameters(dcrf_crf *h, float *out, int capacity, int *n);
int dcrf_set_label_compatibility_parameters(dcrf_crf *h, const float *v, int n);
int dcrf_kernel_parameters(dcrf_crf *h, float *out, int capacity, int *n);
int dcrf_set_kernel_parameters(dcrf_crf *h, const float *v, int n);

/* Number of compatibility and kernel parameters of term `term` in the layout
 * of dcrf_backward: compatibility Potts 1, Diagonal M, Matrix M*M; kernel
 * CONST 0, DIAG d, FULL d*d. */
int dcrf_param_counts(dcrf_crf *h, int term, int *n_compat, int *n_kernel);

/* inference(n) that also keeps every iterate Q_0..Q_T on the device, for
 * dcrf_backward (the per-iteration storage of DenseCRF::gradient,
 * densecrf.cpp:240-253). */
int dcrf_inference_checkpointed(dcrf_crf *h, int n_iterations, float *Q, int layout, int where);

/* Memory of the checkpointed forward: with every = k > 1, only the iterates
 * Q_0, Q_k, Q_2k, ... and Q_T are kept, and dcrf_backward recomputes each
 * k-iteration segment from its first iterate before taking it apart (the
 * recomputed iterates equal the forward's bit for bit).  Iterate storage goes
 * from T+1 rows to T/k + 2 rows plus k+1 for the segment, the per-step lattice
 * and slice storage from T steps to k; the forward's kernels run once more.
 * every = 1 (the default) keeps every iterate, as DenseCRF::gradient does
 * (densecrf.cpp:240-253).  Applies from the next dcrf_inference_checkpointed. */
int dcrf_set_checkpoint_interval(dcrf_crf *h, int every);

/* Adjoint of the last dcrf_inference_checkpointed (DenseCRF::gradient,
 * densecrf.cpp:255-296, for any loss): given dQ = dL/dQ_T (M x N in `layout`,
 * `where`), writes dU = dL/dU (same layout and place; NULL to skip), and, on the
 * HOST, dcompat = dL/d(compatibility values) and dkernel = dL/d(kernel
 * parameters), each the concatenation over terms in dcrf_param_counts order
 * (NULL to skip; kernel gradients cost extra lattice passes).  For a Matrix
 * compatibility the M*M values are dL/dW for the symmetrised W actually used.
 * The lattice filter's transpose is the reverse-order blur
 * (permutohedral.cpp:556). */
int dcrf_backward(dcrf_crf *h, const float *dQ, int layout, int where, float *dU, double *dcompat, double *dkernel);

/* The logistic unary's parameter gradient after dcrf_backward: dL/dL =
 * (dL/dU) f^T, the sum over the iterations of LogisticUnaryEnergy::gradient(b)
 * that DenseCRF::gradient adds (unary.cpp:64-67, densecrf.cpp:292-294), in the
 * order of dcrf_unary_parameters; *n = M * nfeat (0 for a constant unary).
 * Labels M <= 32. */
int dcrf_unary_gradient(dcrf_crf *h, double *out, int capacity, int *n);

/* ---- autotuning (no reference counterpart) --------------------------------
 * The engine's launch and build knobs -- threads per point of the mean-field
 * point pass (1 or 2), its shared-memory budget per CTA (KB), the splat task
 * length (members per task, 1..63), the lattice hash-table load factor, and
 * whether the blur runs all axes in one cooperative launch (1) or one launch
 * per axis (0) --
 * are picked per configuration (labels, per-term d / compatibility kind /
 * normalisation / arithmetic variant, one image or a batch, size class
 * log2 N) by timing candidates on the handle's own lattices.  Choices are
 * remembered for the process.  Only the task length changes results (the
 * grouping of the splat sums, at the 1e-7 level). */

/* Tune at the first inference of every new configuration (or take the
 * remembered choice). Off by default. */
int dcrf_set_autotune(dcrf_crf *h, int on);
/* Tune now for the current terms (rebuilds the lattices while trying). */
int dcrf_autotune(dcrf_crf *h);
/* The knobs in effect (any pointer may be NULL). */
int dcrf_get_tuning(dcrf_crf *h, int *split, int *smem_kb, int *task_len, float *hash_load, int *coop_blur);
/* Set the knobs (split 0 = rule of thumb, smem_kb 0 = default); rebuilds the
 * lattices when the task length or load factor changes. */
int dcrf_set_tuning(dcrf_crf *h, int split, int smem_kb, int task_len, float hash_load, int coop_blur);

/* ---- measurement -------------------------------------------------------- */

/* Number of kernels this library has launched in the process so far. */
int dcrf_launch_count(unsigned long long *count);

/* Kernel classes timed by the profiling mode. */
#define DCRF_KCLASS_POINT 0   /* slice + compatibility + softmax + tile splat */
#define DCRF_KCLASS_REDUCE 1  /* per-vertex sum of the splat partials */
#define DCRF_KCLASS_BLUR 2    /* one blur axis */
#define DCRF_KCLASS_LATTICE 3 /* lattice build (all of its launches) */
#define DCRF_KCLASS_OTHER 4   /* layout conversions, feature generation */
#define DCRF_KCLASS_NORM 5    /* the kernel normalisation of new terms (DenseKernel::initLattice) */
#define DCRF_NUM_KCLASSES 6

/* on = 1: bracket every kernel launch of the handle with CUDA events on its
 * stream (adds a little overhead); 0: off.  Resets the accumulated profile. */
int dcrf_set_profiling(dcrf_crf *h, int on);

/* Accumulated device time (ms, from the events) and launch count of a kernel
 * class since profiling was switched on.  Synchronises the handle's stream. */
int dcrf_profile(dcrf_crf *h, int kernel_class, double *total_ms, long long *launches);

/* Sizes of term `term`: lattice vertices L, splat partials P, tiles. */
int dcrf_term_stats(dcrf_crf *h, int term, int *L, int *P, int *ntiles);

/* ---- introspection (test and debugging aids) ---------------------------- */

/* Number of points, labels and pairwise terms. */
int dcrf_info(dcrf_crf *h, int *N, int *M, int *n_terms);

/* Lattice dimension d and vertex count L of term `term`. */
int dcrf_lattice_info(dcrf_crf *h, int term, int *d, int *L);

/* Copies term `term`'s lattice tables to HOST buffers in the layout of the
 * reference's Permutohedral members (permutohedral.h:49-53): offset, rank and
 * bary as N x (d+1) (point-major), neighbors as (d+1) x L pairs (n1, n2) with
 * -1 for a missing neighbour, keys as L x d int16.  Any pointer may be NULL. */
int dcrf_lattice_dump(dcrf_crf *h, int term, int *offset, int *rank, float *bary, int *neighbors, int16_t *keys);

/* The normalisation vector of term `term` (DenseKernel::norm_,
 * pairwise.cpp:40-62) to a HOST buffer of N floats. */
int dcrf_term_norm(dcrf_crf *h, int term, float *norm);

/* Copies a working buffer of term `term` to a HOST buffer of `count` floats:
 * which = 0 / 1: the two lattice-value buffers ((L+1) rows of the padded label
 * count; row 0 is the zero sentinel); 2: the per-tile splat partials. */
int dcrf_term_buffer(dcrf_crf *h, int term, int which, float *out, size_t count);

/* Lattice filter of term `term` alone (Permutohedral::compute,
 * permutohedral.cpp:596-604): out = K in for value_size rows, both
 * (value_size, N) label-major on the HOST; reverse = transposed (reverse-order
 * blur).  value_size must equal 1 or the handle's M. */
int dcrf_lattice_filter(dcrf_crf *h, int term, const float *in, int value_size, int reverse, float *out);

/* ---- allocation-free variant ---------------------------------------------- */

/* Maximum scratch of dcrf_lattice_filter_noalloc, in floats (32 MiB), held in a
 * static device array by every GPU that loads the library, until exit. */
#define DCRF_NOALLOC_MAX_FLOATS (8u * 1024u * 1024u)

/* The raw lattice filter of dcrf_lattice_filter, for callers that must not
 * allocate device memory while they run: code working inside a fixed memory
 * budget owned by another allocator (a framework's caching allocator, a
 * serving runtime), or a pipeline that forbids cudaMalloc/cudaFree after
 * start-up because they synchronise the device and take unbounded time.  It
 * calls no cudaMalloc, cudaFree or allocating library routine: its scratch is
 * one static device array of DCRF_NOALLOC_MAX_FLOATS floats.  Term `term` must
 * already be built (dcrf_add_pairwise*).
 *   in, out: DEVICE pointers, (value_size, N) label-major; value_size is 1 or M.
 *            `in` must be ready, and both must stay valid, in `stream`'s order.
 *   stream:  cudaStream_t the work is ordered on (NULL: the legacy default
 *            stream); the call returns once the work is enqueued.  The work
 *            starts after everything already queued on the handle's stream
 *            (dcrf_set_stream; a term's build finishes there after
 *            dcrf_add_pairwise* returns), and the handle's stream waits for it
 *            before its own later work, through an event the handle created at
 *            dcrf_create*.  Passing the handle's stream is fine.
 * A bounded device wait that gives up inside this call is recorded in the
 * handle's status block and returned by the handle's next synchronising call
 * (dcrf_synchronize, an inference, a build).
 * The first call on a device resolves the array's address on that device
 * (cudaGetSymbolAddress) and should come before any stream capture.  All calls
 * share the one array and it keeps the last call's contents: calls that may
 * overlap on the GPU (other streams, other host threads) race and must be
 * serialised by the caller.  A problem whose scratch exceeds the maximum
 * (slots*P + (partials+1)*P + 2*(vertices+1)*P floats, P the padded value
 * size up to 32; more labels are filtered 32 at a time through the same
 * scratch, P = 32) is rejected with DCRF_ERR_INVALID_ARG.
 * No counterpart in the reference (added for allocation-free callers). */
int dcrf_lattice_filter_noalloc(dcrf_crf *h, int term, const float *in, int value_size, int reverse, float *out,
                                void *stream);

/* Failure-detection check of the device-side bounded waits.  Launches, on the
 * handle's stream, one warp that waits on a device flag nothing sets, giving up
 * after `spins` polls (1..1048576, each followed by a ~256 ns sleep) the way the
 * point pass's copy barrier and the cooperative blur's grid barrier give up: it
 * records DCRF_ERR_TIMEOUT in the handle's device status block and returns.
 * The call synchronises and returns that status (DCRF_ERR_TIMEOUT expected;
 * anything else means the wait or the status path is broken); the status is
 * cleared and the handle stays usable.
 * No counterpart in the reference (a diagnostic of this engine). */
int dcrf_check_bounded_wait(dcrf_crf *h, int spins);

#ifdef __cplusplus
}
#endif
#endif /* DCRF_GB300_H */
