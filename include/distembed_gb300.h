/*
 * distembed_gb300 — C ABI of the GPU force-model SGD graph-embedding step.
 *
 * This library replaces the one-rank branch of DistEmbed's
 *   template<INDEX_TYPE, VALUE_TYPE, embedding_dim> class EmbeddingAlgo
 *     EmbeddingAlgo(SpMat* native, SpMat* receiver, SpMat* sender, DenseMat* dense,
 *                   Process3DGrid* grid, double alpha, double beta,
 *                   VALUE_TYPE MAX_BOUND, VALUE_TYPE MIN_BOUND, bool col_major, bool sync_comm)
 *                                                             (cpp/algo/algo.hpp:54-63)
 *     void algo_force2_vec_ns(int iterations, int batch_size, int ns, VALUE_TYPE lr)
 *                                                             (cpp/algo/algo.hpp:74-262)
 * behind plain pointers and sizes.  The graph and the embedding stay resident on
 * one GPU between calls; nothing is partitioned and no collective runs.
 *
 * Data handed across (the same arrays the reference algo reads):
 *   CSR      rowptr[n+1], col[nnz]  int64, as CSRHandle::rowStart / col_idx
 *            (cpp/core/common.h:127-131), columns ascending within a row
 *   x        n x dim row-major FP64, as DenseMat::nCoordinates (cpp/core/dense_mat.hpp:34)
 *
 * Every entry point returns DE_OK (0) or a negative DE_ERR_* code; the text of
 * the last error of a handle is available from de_last_error().  A handle is
 * used from one host thread at a time; all its GPU work runs on one stream.
 */
#ifndef DISTEMBED_GB300_H
#define DISTEMBED_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DE_OK 0
#define DE_ERR_INVALID (-1)     /* bad argument or unsupported shape            */
#define DE_ERR_OOM (-2)         /* device or pinned host allocation failed      */
#define DE_ERR_CUDA (-3)        /* CUDA runtime or kernel error                 */
#define DE_ERR_STATE (-4)       /* call out of order (e.g. run before set)      */
#define DE_ERR_UNSUPPORTED (-5) /* valid request this build cannot serve        */

#define DE_PRECISION_FP32 0 /* FP32 embedding, FP32 arithmetic                   */
#define DE_PRECISION_BF16 1 /* BF16 storage, FP32 master copy and accumulation  */

typedef struct de_handle de_handle;

typedef struct de_options {
  int32_t precision;    /* DE_PRECISION_*                                              */
  int32_t ref_quirks;   /* 1: reproduce the reference's one-rank behaviour exactly:    */
                        /*    edges into vertex n-1 are skipped (algo.hpp:399-405,538) */
                        /*    and from the second epoch of a call the repulsive pass   */
                        /*    covers last_batch_size rows (algo.hpp:135,167-169,594)   */
  int32_t compute_loss; /* 1: accumulate the FP64 per-epoch loss                       */
  int32_t device;       /* CUDA device ordinal                                         */
  void *stream;         /* cudaStream_t to run on; NULL: the handle creates its own    */
  double max_bound;     /* clip bound of every force component (reference: 5)          */
  int32_t edge_cap;     /* max CSR entries per work item (1..32); 0 = automatic        */
  int32_t pdl;          /* 1: overlap consecutive minibatch launches (programmatic     */
                        /*    dependent launch); 0: plain stream order                 */
  int32_t stage_negatives; /* FP32 plain form, ns <= 8: 1 copies the minibatch's      */
                        /*    negative rows into each CTA's shared memory (bulk async  */
                        /*    copy) before the repulsive pass; 0 reads them from L1/L2 */
  int32_t reserved[5];
} de_options;

/* Fills *o with the defaults: FP32, quirks on, loss on, device 0, own stream, bound 5,
 * automatic edge cap, programmatic dependent launch on, negatives read from L1/L2
 * (the shared-memory staging measured 8.5% slower at R-MAT scale 20). */
void de_default_options(de_options *o);

/* Uploads the CSR (n vertices, nnz entries) and prepares a handle for embeddings of
 * width dim (32, 64, 128 or 256).  Replaces the EmbeddingAlgo constructor
 * (cpp/algo/algo.hpp:54-63) together with the CSR build it reads
 * (cpp/core/csr_local.hpp:37-125).  The embedding starts at zero. */
int de_create(int64_t n, const int64_t *rowptr, const int64_t *col, int64_t nnz, int32_t dim,
              const de_options *opts, de_handle **out);

/* Frees every device and host resource of the handle.  NULL is accepted. */
int de_destroy(de_handle *h);

/* Host FP64 n x dim row-major in/out, the layout of DenseMat::nCoordinates. */
int de_set_embeddings(de_handle *h, const double *x);
int de_get_embeddings(de_handle *h, double *x);

/* FP32 n x dim row-major in/out; on_device = 1 when x is a device pointer. */
int de_set_embeddings_f32(de_handle *h, const float *x, int32_t on_device);
int de_get_embeddings_f32(de_handle *h, float *x, int32_t on_device);

/* Runs `epochs` epochs of minibatch force-model SGD on the resident embedding:
 * the body of EmbeddingAlgo::algo_force2_vec_ns (cpp/algo/algo.hpp:74-262) at one
 * rank.  lr_per_epoch[epochs] holds one rate per epoch (the reference uses one
 * constant rate).  Negatives are drawn exactly as the reference draws them
 * (seed = epoch + batch, cpp/algo/algo.hpp:165-173, cpp/core/common.cpp:37-53).
 * loss_per_epoch (nullable): when given, the call waits for the GPU and writes the
 * FP64 loss of each epoch.  When NULL the call returns once the work is queued. */
int de_run(de_handle *h, int32_t epochs, int32_t batch_size, int32_t ns,
           const double *lr_per_epoch, double *loss_per_epoch);

/* de_run resumed at epoch `first_epoch` of a call: epoch i of this call uses the
 * seeds and the repulsive row count of epoch first_epoch + i, so running epochs
 * [0, a) and then [a, b) equals one de_run of b epochs.  lr_per_epoch and
 * loss_per_epoch are indexed from 0 (the first epoch run here).  The reference
 * has no resume; this is the checkpoint/restart entry (state = embedding + epoch). */
int de_run_from(de_handle *h, int32_t first_epoch, int32_t epochs, int32_t batch_size, int32_t ns,
                const double *lr_per_epoch, double *loss_per_epoch);

/* Runs one epoch (epoch first_epoch of a call, one learning rate) like de_run_from,
 * but launches its kernels one by one with CUDA events between them and waits:
 * launch_ms[i] is the device time of launch i and launch_kind[i] its kind (0: the
 * minibatch kernel of the FP32 form / the attractive kernel of the BF16 form,
 * 1: BF16 repulsion GEMM kernel, 2: BF16 update with the exact close pairs,
 * 3: epoch flush, 4: BF16 negative gather); the launches of the profiled epoch
 * run one after another (the BF16 attractive pass and GEMMs are not overlapped).
 * *count receives the number of launches; capacity must be at least that.  The
 * epoch is a real step: the embedding is updated.  No reference counterpart:
 * this is the per-kernel timing used by the benchmark. */
int de_profile_epoch(de_handle *h, int32_t first_epoch, int32_t batch_size, int32_t ns, double lr,
                     float *launch_ms, int32_t *launch_kind, int32_t capacity, int32_t *count);

/* Waits for all queued work of the handle. */
int de_sync(de_handle *h);

/* Number of edge-updates (attractive (vertex, neighbour) plus repulsive
 * (vertex, negative) force evaluations) that de_run_from with these arguments
 * performs.  Negative on a bad argument. */
int64_t de_edge_updates(de_handle *h, int32_t first_epoch, int32_t epochs, int32_t batch_size,
                        int32_t ns);

/* The reference's negative sampler: ns draws of uniform_int_distribution<int>(0, n)
 * from minstd_rand(seed) (cpp/core/common.cpp:37-53), on the host. */
void de_negatives(int64_t n, int32_t seed, int32_t ns, int64_t *out);

/* One minibatch of the FP32 plain step on caller-owned device memory, allocating
 * nothing.  No counterpart in the reference: it exists for callers that may not
 * allocate device memory (a host framework that owns the device heap through its
 * own pool, a latency-bound loop that cannot take cudaMalloc's implicit device
 * synchronisation).  All pointers are device pointers: rowptr[n+1] and col (int32
 * CSR), x (n x dim FP32, updated in place for rows of the minibatch), negs[ns]
 * (this minibatch's draws), loss (nullable, one FP64: this minibatch's loss).
 * rep_rows: leading rows of the minibatch that take the repulsive pass;
 * skip_last_vertex: 1 drops edges into vertex n-1 as the reference does.  Work
 * memory is a fixed device array of the library: batch rows * dim <= 1,048,576.
 * Larger minibatches return DE_ERR_INVALID (text in de_last_error(NULL)).  Every
 * call looks that array's address up in the current context
 * (cudaGetSymbolAddress), so a new context after a device reset is followed; the
 * first call on a device also loads the module, so make it before any stream
 * capture.  Calls share the array: calls that overlap on the GPU race.  Launches on `stream` (a cudaStream_t, NULL = default stream) and
 * returns without waiting. */
int de_minibatch_noalloc(int64_t n, const int32_t *rowptr, const int32_t *col, int32_t dim, float *x,
                         int32_t batch_id, int32_t batch_size, const int32_t *negs, int32_t ns,
                         int32_t rep_rows, int32_t skip_last_vertex, float lr, float max_bound,
                         double *loss, void *stream);

/* ---- Batched form: many independent graphs trained in one persistent launch.
 * No counterpart in the reference, which trains one graph per process
 * (cpp/dist_embed.cpp:334-344 builds one EmbeddingAlgo and calls
 * algo_force2_vec_ns once); each graph here follows that same one-rank step
 * (cpp/algo/algo.hpp:164-192) with its own sampler seeds (epoch + batch), as if
 * it ran alone.  One CTA ("team") owns a graph for all its epochs; teams take
 * graphs largest first.  dim is 32, 64 or 128; opts->precision picks FP32
 * storage or BF16 storage with an FP32 master copy; opts->edge_cap (0: 32) is the
 * CSR entries of one work item, up to 4096. */
typedef struct de_batch de_batch;

/* Graph g has n[g] vertices and CSR rowptr[g][n[g]+1], col[g][rowptr[g][n[g]]]
 * (local vertex ids).  Embeddings start at zero: set them before running. */
int de_batch_create(int32_t n_graphs, const int64_t *n, const int64_t *const *rowptr,
                    const int64_t *const *col, int32_t dim, const de_options *opts, de_batch **out);
int de_batch_destroy(de_batch *b);
/* Host FP32 (n[g] x dim) embedding of graph g in / out; graph = -1: every graph's,
 * concatenated in graph order (sum of n x dim). */
int de_batch_set_embeddings_f32(de_batch *b, int32_t graph, const float *x);
int de_batch_get_embeddings_f32(de_batch *b, int32_t graph, float *x);
/* Team shape.  Two kernel families run the same step:
 *   DE_BATCH_REGISTER  work items read their rows into registers; a warp runs
 *                      vertices_per_warp (1, 2 or 4) items at once on 32, 16 or 8
 *                      lanes; team_warps 4, 8, 16 or 32; edge_cap 1..4096
 *   DE_BATCH_STAGED    every warp stages the rows of its next stages-1 chunks in
 *                      shared memory with 16-byte asynchronous copies; a pair is
 *                      computed by dim/8 lanes; team_warps 2..16; edge_cap 1..32
 *                      (one chunk); pairs = warp steps in flight (1 or 2);
 *                      stages 3 or 4 ring slots per warp; at most 32 negatives
 *                      per minibatch
 *   DE_BATCH_ROWS      the staged pipeline with one work item per group of
 *                      dim/8 lanes (32/(dim/8) items per warp chunk); same
 *                      fields as DE_BATCH_STAGED
 * A shape that does not exist for the batch's dim returns DE_ERR_UNSUPPORTED. */
#define DE_BATCH_REGISTER 0
#define DE_BATCH_STAGED 1
#define DE_BATCH_ROWS 2
typedef struct de_batch_shape {
  int32_t kernel;            /* DE_BATCH_*                                   */
  int32_t vertices_per_warp; /* register kernel                              */
  int32_t team_warps;        /* warps per team (one CTA per team)            */
  int32_t edge_cap;          /* CSR entries per work item                    */
  int32_t pairs;             /* staged kernel: warp steps in flight          */
  int32_t stages;            /* staged kernel                                */
  int32_t team_ctas;         /* staged kernel: 2 or 4 = the largest graphs    */
                             /* are trained by the CTAs of a cluster of that  */
                             /* size together (the rest one per CTA); 0 or 1  */
                             /* = one CTA each                                */
} de_batch_shape;
int de_batch_set_shape(de_batch *b, const de_batch_shape *shape);
int de_batch_get_shape(const de_batch *b, de_batch_shape *shape);
/* Trains every graph for `epochs` epochs (minibatch batch_size, ns shared
 * negatives per minibatch, lr_per_epoch[epochs]) in one launch captured in a CUDA
 * graph, and waits.  loss (nullable): [n_graphs x epochs] FP64 per-graph epoch
 * loss. */
int de_batch_run(de_batch *b, int32_t epochs, int32_t batch_size, int32_t ns, const double *lr_per_epoch,
                 double *loss);
/* de_batch_run in three parts.  prepare: builds the work lists, draws the
 * negatives, allocates the team staging areas and captures the one launch in a
 * CUDA graph (host work; nothing runs).  launch: replays that graph on the batch's
 * stream and returns; every launch trains every graph for the prepared epochs
 * again, from the embeddings it finds.  wait: waits for the stream and, when
 * loss is given, copies the [n_graphs x epochs] loss of the last launch. */
int de_batch_prepare(de_batch *b, int32_t epochs, int32_t batch_size, int32_t ns, const double *lr_per_epoch);
int de_batch_launch(de_batch *b);
int de_batch_wait(de_batch *b, double *loss);
/* Times every team shape of both kernel families on `epochs` epochs of the real
 * workload, keeps the fastest (de_batch_set_shape) and leaves the embeddings as
 * they were.  ms / shapes (nullable, capacity entries): the time and the shape of
 * each one tried, in the order tried; *count (nullable): how many were tried;
 * *best (nullable): the shape kept. */
int de_batch_autotune(de_batch *b, int32_t epochs, int32_t batch_size, int32_t ns, double lr, float *ms,
                      de_batch_shape *shapes, int32_t capacity, int32_t *count, de_batch_shape *best);
/* BF16 form: a pair whose squared distance computed from the BF16 copies is below
 * near_r (default 0.02) is read again from the FP32 master and recomputed; 0 turns
 * this off.  Close pairs are the ones whose distance the BF16 rounding step
 * distorts. */
int de_batch_set_near_distance(de_batch *b, float near_r);
/* Which epochs of a run compute their FP64 loss (the reference computes none):
 * DE_LOSS_EVERY_EPOCH (default), DE_LOSS_LAST_EPOCH (only the last epoch of each
 * run; the others report 0, and their passes take no logarithm) or DE_LOSS_NONE.
 * Takes effect at the next de_batch_prepare / de_batch_run. */
#define DE_LOSS_NONE 0
#define DE_LOSS_EVERY_EPOCH 1
#define DE_LOSS_LAST_EPOCH 2
int de_batch_set_loss(de_batch *b, int32_t mode);
/* Per graph of the last launch: {start, end} (globaltimer ns) and the team that
 * ran it; out holds n_graphs x 3 values.  Waits for the stream. */
int de_batch_trace(de_batch *b, int64_t *out);
/* Edge-updates de_batch_run performs with these arguments, summed over graphs. */
int64_t de_batch_edge_updates(de_batch *b, int32_t epochs, int32_t batch_size, int32_t ns);
/* The cudaStream_t the batch runs on (as void*). */
void *de_batch_stream(de_batch *b);
/* Text of the last error on b (NULL: of the last failed de_batch_create). */
const char *de_batch_last_error(const de_batch *b);

/* ---- Served form: a request loop that trains embedding jobs concurrently.
 * No counterpart in the reference, which runs one job per process
 * (cpp/dist_embed.cpp:156-347).  Each job is the one-rank step of
 * cpp/algo/algo.hpp:164-192 on its own resident handle (FP32 plain or BF16
 * form), so its result is the same alone or among other jobs.  Jobs are
 * admitted in submission order when one of `slots` worker slots is free and the
 * job's device footprint fits in the memory budget; every slot has its own CUDA
 * stream, so the running jobs' kernels share the GPU and a job that arrives
 * while others run starts as soon as a slot and memory free up. */
typedef struct de_server de_server;

#define DE_JOB_QUEUED 0
#define DE_JOB_RUNNING 1
#define DE_JOB_DONE 2
#define DE_JOB_FAILED 3

/* A job.  The arrays are the caller's and must stay valid (and x0, rowptr, col
 * unchanged) until de_server_wait returns for the job. */
typedef struct de_job_spec {
  int64_t n;                  /* vertices                                        */
  const int64_t *rowptr;      /* [n+1] CSR, columns ascending within a row       */
  const int64_t *col;         /* [nnz]                                           */
  int64_t nnz;
  int32_t dim;                /* 32, 64, 128 or 256 (BF16: 64..256)              */
  int32_t precision;          /* DE_PRECISION_*                                  */
  int32_t epochs, batch_size, ns;
  int32_t pad;
  const double *lr_per_epoch; /* [epochs]                                        */
  const float *x0;            /* [n x dim] FP32 start embedding                  */
  float *x_out;               /* [n x dim] FP32 result                           */
  double *loss_out;           /* nullable: [epochs] FP64 loss per epoch          */
} de_job_spec;

typedef struct de_job_info {
  int32_t state;              /* DE_JOB_*                                        */
  int32_t pad;
  double submit_s, start_s, end_s; /* server clock (de_server_clock), seconds   */
  int64_t device_bytes;       /* memory reserved for the job                     */
  int64_t edge_updates;       /* force evaluations the job performs              */
} de_job_info;

typedef struct de_server_stats {
  int64_t submitted, done, failed, queued, running, peak_running;
  int64_t budget_bytes, reserved_bytes, peak_reserved_bytes;
} de_server_stats;

/* slots: jobs in flight at most.  Memory budget: hbm_bytes when > 0, else
 * hbm_fraction (0 < f <= 1; 0: 0.8) of the device's free memory at creation,
 * allocated once.  ref_quirks as in de_options. */
int de_server_create(int32_t device, int32_t slots, int64_t hbm_bytes, double hbm_fraction, int32_t ref_quirks,
                     de_server **out);
/* Queues a job; *id identifies it.  A job larger than the whole budget returns
 * DE_ERR_UNSUPPORTED. */
int de_server_submit(de_server *s, const de_job_spec *job, int64_t *id);
/* Current state of a job that has not been waited for. */
int de_server_info(de_server *s, int64_t id, de_job_info *info);
/* Waits until the job is done (x_out and loss_out written), returns its info
 * and forgets it. */
int de_server_wait(de_server *s, int64_t id, de_job_info *info);
/* Waits until no job is queued or running. */
int de_server_drain(de_server *s);
int de_server_get_stats(de_server *s, de_server_stats *stats);
/* Seconds since the server was created (the clock of de_job_info). */
double de_server_clock(const de_server *s);
/* Finishes the queued jobs, stops the slots and frees the budget. */
int de_server_destroy(de_server *s);
const char *de_server_last_error(const de_server *s);

/* ---- Input and output of the driver (de_mm_read and the writer: host only).
 * MatrixMarket reader with the semantics of ParallelIO::parallel_read_MM
 * (cpp/io/parrallel_IO.hpp:31-88) at one rank: coordinate format, 1-based,
 * duplicates merged, values ignored, a symmetric header mirrors off-diagonal
 * entries; CSR columns ascending.  Call with rowptr = col = NULL for the sizes
 * (rows, cols, nnz after merging), then with rowptr[rows+1], col[capacity >= nnz]. */
int de_mm_read(const char *path, int64_t *rows, int64_t *cols, int64_t *nnz, int64_t *rowptr, int64_t *col,
               int64_t capacity);
/* The same reader with the COO -> CSR (sort of the entries, merge of duplicates,
 * row pointers) on GPU `device`: the file is parsed on the host once, the CSR is
 * the one de_mm_read returns.  The result is read through de_csr_info /
 * de_csr_copy and released with de_csr_free. */
typedef struct de_csr de_csr;
int de_mm_read_gpu(const char *path, int32_t device, de_csr **out);
/* COO -> CSR on GPU `device` for 0-based entries (row_idx[e], col_idx[e]) of a
 * rows x cols matrix, with the mirrored entry of every off-diagonal one when
 * mirror != 0; duplicates merged, columns ascending within a row
 * (cpp/core/csr_local.hpp:37-125 at one rank, MKL's order defined as ascending). */
int de_coo_to_csr(int64_t rows, int64_t cols, const int64_t *row_idx, const int64_t *col_idx, int64_t nnz,
                  int32_t mirror, int32_t device, de_csr **out);
int de_csr_info(const de_csr *c, int64_t *rows, int64_t *cols, int64_t *nnz);
/* rowptr[rows + 1], col[nnz]. */
int de_csr_copy(const de_csr *c, int64_t *rowptr, int64_t *col);
void de_csr_free(de_csr *c);
/* Embedding writer of ParallelIO::parallel_write (cpp/io/parrallel_IO.hpp:90-146):
 * per row "%lu" (1-based id), dim times " %.5f", "\n"; no header. */
int de_embedding_write(const char *path, const double *x, int64_t rows, int32_t dim);

/* SpMMAlgo::algo_spmm(1, batch_size, lr) at one rank (cpp/algo/spmm.hpp:54-159),
 * as BaselineSpMM::execute runs it for -spmm 1 (cpp/algo/baseline_spmm.hpp:63-88):
 * y = lr * A x for the handle's CSR and current embedding x, minibatch by
 * minibatch (the rows do not depend on one another; x is not changed); with
 * ref_quirks edges into vertex n-1 are skipped (spmm.hpp:260-265, 365).
 * y: host FP64 n x dim (the output DenseMat's layout). */
int de_spmm(de_handle *h, int32_t batch_size, double lr, double *y);
/* The same into an FP32 n x dim buffer (a device pointer when on_device). */
int de_spmm_f32(de_handle *h, int32_t batch_size, float lr, float *y, int32_t on_device);

/* SparseEmbedding::algo_sparse_embedding(iterations, batch_size, ns, lr, density)
 * at one rank (cpp/algo/sparse_embedding.hpp:78-194), which the driver runs for
 * -sparse_embedding 1 (cpp/dist_embed.cpp:317-330).  x: host FP64 n x dim rows in
 * the reference's dense-collector form, INT_MIN marking an absent entry
 * (cpp/core/sparse_mat.hpp:367-377, 492-505); replaced by the rows after the
 * run, absent entries as 0.  k = (int)(dim * density).
 *   merge = 0: the reference's one-rank branch (lines 138-144).  The attractive
 *     force on the union of two rows' present entries (lines 338-503) goes into
 *     the batch collector, which that branch never merges: the values change
 *     only by the top-k pruning after the first iteration (lines 172-186,
 *     745-767).  coll (host FP64 batch_size x dim, may be NULL) receives the
 *     collector: slot r summed over rows r, B + r, ... of every iteration.
 *   merge = 1: per minibatch the repulsive pass on its negatives (lines 505-659),
 *     the attractive pass, then merge_batch_collector (sparse_mat.hpp:385-400):
 *     the steps of the multi-rank branch (lines 145-168) that touch the local
 *     partition, with the repulsive row count of F8 under ref_quirks; the rows are
 *     pruned to their k largest values after every iteration but the last.
 * At equal values the pruning drops the lower dim first (the reference's heap
 * order at ties is its own).  The handle's FP32 embedding becomes the rows'
 * FP32 mirror (0 for an absent entry).  FP32 handles, dim 32, 64, 128 or 256. */
int de_sparse_embedding(de_handle *h, double *x, int32_t iterations, int32_t batch_size, int32_t ns, double lr,
                        double density, int32_t merge, double *coll);
/* The same in three steps, the rows kept on the device between them:
 * de_sparse_set copies x (host or device memory) in, de_sparse_run enqueues the run on the handle's
 * stream (returns before it completes), de_sparse_get waits and copies the rows
 * (n x dim) and/or the collector (the last run's batch_size x dim); either may
 * be NULL. */
int de_sparse_set(de_handle *h, const double *x);
int de_sparse_run(de_handle *h, int32_t iterations, int32_t batch_size, int32_t ns, double lr, double density,
                  int32_t merge);
int de_sparse_get(de_handle *h, double *x, double *coll);

/* The cudaStream_t the handle runs on (as void*). */
void *de_stream(de_handle *h);

/* Text of the last error on h (or of the last failed de_create when h is NULL). */
const char *de_last_error(const de_handle *h);

/* Library version string. */
const char *de_version(void);

#ifdef __cplusplus
}
#endif

#endif /* DISTEMBED_GB300_H */
