/*
 * yell_gb300 — C ABI of the GB300 (sm_103a) implementation of YELL's RNS
 * polynomial hot path: negacyclic forward / inverse NTT over 62-bit primes,
 * pointwise Barrett mulmod, muladd, add/sub, negate and a fused polymul.
 *
 * Every entry point returns an int status (0 = YELL_OK) and never aborts;
 * yell_last_error() gives a thread-local message for the last failure.
 * Plain pointers and sizes only.  Residues are uint64 words; "limb" cm of a
 * polynomial is reduced modulo prime yell_prime(cm) exactly as in the
 * reference, where limb cm of yell::poly<N> uses params::P[cm]
 * (include/yell/details/poly.hpp:170-186).
 *
 * Results are word-for-word those of the reference (fionser/YELL) on the
 * same inputs: forward outputs in bit-reversed order, reduced to [0, p)
 * (forward) or left in [0, 4p) (forward_lazy, the same lazy words as the
 * reference); backward outputs in natural order in [0, p).
 *
 * Degrees: N = 2^log_n with log_n in [3, 20] (yell_min_log_degree() ..
 * yell_max_log_degree()).  The reference's inverse at N = 4 applies its last
 * layer twice (lib/ntt.cpp:174-187 followed by
 * include/yell/details/ntt.hpp:144-159) and is not an inverse, so 4 is
 * rejected with YELL_ERR_UNSUPPORTED_DEGREE.
 *
 * Three families of calls:
 *   1. Drop-ins for the reference's host-memory calls (yell_ntt_*,
 *      yell_poly_*): host pointers, copied to the GPU and back inside the
 *      call.  Synchronous.
 *   2. Device-resident calls (yell_dev_*): device pointers owned by the
 *      caller, work queued on the given CUDA stream (NULL = the library's
 *      stream of the current device), asynchronous.
 *   3. Handles (yell_dev_poly_*), a batch queue (yell_batch_*) and a serving
 *      loop (yell_server_*) built on 2.
 */
#ifndef YELL_GB300_H_
#define YELL_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define YELL_GB300_ABI_VERSION 1

enum yell_status_code {
  YELL_OK = 0,
  YELL_ERR_INVALID_ARGUMENT = 1,   /* null pointer, zero count, bad enum */
  YELL_ERR_UNSUPPORTED_DEGREE = 2, /* log_n outside [3, 20] */
  YELL_ERR_INVALID_MODULUS = 3,    /* cm >= yell_max_moduli() */
  YELL_ERR_CUDA = 4,               /* a CUDA call failed; see yell_last_error() */
  YELL_ERR_OUT_OF_MEMORY = 5,      /* device or pinned allocation refused */
  YELL_ERR_BUDGET = 6,             /* request exceeds the server's HBM budget */
  YELL_ERR_TIMEOUT = 7,            /* a bounded wait gave up */
  YELL_ERR_CANCELLED = 8,          /* request cancelled before it ran */
  YELL_ERR_NOT_FOUND = 9,          /* unknown request id */
  YELL_ERR_NO_DEVICE = 10          /* no CUDA device visible */
};

enum yell_direction { YELL_FORWARD = 0, YELL_FORWARD_LAZY = 1, YELL_BACKWARD = 2 };

enum yell_elementwise_op {
  YELL_OP_MULMOD = 0, /* dst = mulmod(a, b)            include/yell/ops.hpp:103-112 */
  YELL_OP_ADDMOD = 1, /* dst = addmod(a, b)            include/yell/ops.hpp:54-68   */
  YELL_OP_SUBMOD = 2, /* dst = submod(a, b)            include/yell/ops.hpp:70-83   */
  YELL_OP_MULADD = 3, /* dst = barrett(a*b + dst)      include/yell/ops.hpp:144-158 */
  YELL_OP_NEGATE = 4  /* dst = p - a (b unused)        include/yell/details/poly.hpp:151-157 */
};

/* ---- library --------------------------------------------------------- */
int yell_abi_version(void);
const char* yell_status_string(int status);
const char* yell_last_error(void);
/* Number of kernels this library launched so far in this process. */
uint64_t yell_kernel_launches(void);
/* Device, pinned-host and memory-pool allocations the library has made in
 * this process (no counterpart in the reference): a caller that must not
 * allocate can read it around a call. */
uint64_t yell_allocations(void);

/* ---- params: replaces yell::params (include/yell/params_64.hpp:19-38) --- */
uint32_t yell_max_moduli(void);       /* kMaxNbModuli = 1000 (params_64.hpp:19) */
uint32_t yell_min_log_degree(void);
uint32_t yell_max_log_degree(void);
uint64_t yell_prime(uint32_t cm);          /* params::P[cm], 0 if out of range (:27) */
uint64_t yell_prime_pn(uint32_t cm);       /* params::Pn[cm] (:31)                   */
uint64_t yell_primitive_root(uint32_t cm); /* params::primitive_roots[cm] (:34)      */

/* ---- twiddle tables: replaces ntt<N>::init_table / init_ntt_tables -----
 * (include/yell/ntt.hpp:50-56, include/yell/details/ntt.hpp:28-104).  Tables
 * live on the current device for the life of the process, like the
 * reference's per-N singleton.  Other calls build them on first use; calling
 * these first keeps table construction out of later timed or captured work. */
int yell_init_table(uint32_t log_n, uint32_t cm);
int yell_init_ntt_tables(uint32_t log_n, uint32_t K); /* cm = 0 .. K-1 */
int yell_init_ntt_tables_range(uint32_t log_n, uint32_t cm0, uint32_t L); /* cm0 .. cm0+L-1 */
/* Host copy of one table: out4n = phiTbl, shoupPhiTbl, invphiTbl,
 * shoupInvphiTbl (N words each, bit-reversed); scalars4 = invDegree,
 * shoupInvDegree, invphiInvDegree, shoupInvphiInvDegree (include/yell/ntt.hpp:35-43). */
int yell_ntt_tables(uint32_t log_n, uint32_t cm, uint64_t* out4n, uint64_t* scalars4);

/* ---- drop-in, one limb in host memory, in place -------------------------
 * Replace yell::ntt<N>::forward / forward_lazy / backward(T* op, size_t cm)
 * (include/yell/ntt.hpp:59-65; include/yell/details/ntt.hpp:106-166). */
int yell_ntt_forward(uint64_t* op, uint32_t log_n, uint32_t cm);
int yell_ntt_forward_lazy(uint64_t* op, uint32_t log_n, uint32_t cm);
int yell_ntt_backward(uint64_t* op, uint32_t log_n, uint32_t cm);

/* ---- runtime-N free functions: negacylic_forward_lazy / negacylic_backward_lazy
 * (include/yell/details/ntt.hpp:10-23, lib/ntt.cpp:89-210): in place on host
 * memory, any power-of-two degree 4 .. 2^20, caller-supplied bit-reversed
 * twiddles w and their Shoup companions wshoup (degree words each), p < 2^62.
 * Forward: all log N CT stages, [0,4p) in and out.  Backward: the GS stages
 * except the last layer (m = 1) for N >= 8, as the reference leaves it to its
 * caller.  Drop-ins (one CTA per call), not the batched path. */
int yell_negacyclic_forward_lazy(uint64_t* x, uint64_t degree, const uint64_t* w, const uint64_t* wshoup,
                                 uint64_t p);
int yell_negacyclic_backward_lazy(uint64_t* x, uint64_t degree, const uint64_t* w, const uint64_t* wshoup,
                                  uint64_t p);

/* ---- drop-in, one poly in host memory -----------------------------------
 * limbs = poly<N>::raw_data(): L separate arrays of N words, limb cm using
 * prime cm.  Replace poly<N>::forward / forward_lazy / backward
 * (include/yell/details/poly.hpp:170-186). */
int yell_poly_forward(uint64_t* const* limbs, uint32_t L, uint32_t log_n);
int yell_poly_forward_lazy(uint64_t* const* limbs, uint32_t L, uint32_t log_n);
int yell_poly_backward(uint64_t* const* limbs, uint32_t L, uint32_t log_n);
/* Replace the YELL_BINARY_OPERATOR / YELL_SELF_BINARY_OPERATOR loops
 * (include/yell/ops.hpp:7-41) behind poly<N>::operator* + - *= += -=
 * (include/yell/poly.hpp:163-168).  dst may alias a or b. */
int yell_poly_mulmod(uint64_t* const* dst, const uint64_t* const* a, const uint64_t* const* b,
                     uint32_t L, uint32_t log_n);
int yell_poly_addmod(uint64_t* const* dst, const uint64_t* const* a, const uint64_t* const* b,
                     uint32_t L, uint32_t log_n);
int yell_poly_submod(uint64_t* const* dst, const uint64_t* const* a, const uint64_t* const* b,
                     uint32_t L, uint32_t log_n);
/* Replaces poly<N>::add_product_of: acc += a*b via ops::muladd
 * (include/yell/details/poly.hpp:118-132). */
int yell_poly_add_product_of(uint64_t* const* acc, const uint64_t* const* a,
                             const uint64_t* const* b, uint32_t L, uint32_t log_n);
/* Replaces poly<N>::negate (include/yell/details/poly.hpp:151-157). */
int yell_poly_negate(uint64_t* const* limbs, uint32_t L, uint32_t log_n);

/* ---- fused polymul on host memory ---------------------------------------
 * c = a * b mod (X^N + 1) for `pairs` independent pairs laid out
 * (pairs, L, N) contiguous, limb l using prime cm0 + l: the reference's
 * a.forward(); b.forward(); c = a * b; c.backward(); per pair, fused on the
 * GPU, with host<->device copies pipelined against the compute.  a and b are
 * not modified.  Pinned host memory (yell_host_alloc) copies fastest. */
int yell_polymul_host(uint64_t* c, const uint64_t* a, const uint64_t* b, uint32_t pairs,
                      uint32_t L, uint32_t log_n, uint32_t cm0);
void* yell_host_alloc(size_t bytes); /* pinned; NULL on failure */
void yell_host_free(void* p);

/* Host-pointer calls above 2^15 words (yell_ntt_*, yell_poly_*) on a device
 * that reaches pageable host memory through the host's page tables (GB300
 * with Grace over NVLink-C2C) move the caller's limbs with kernels that load
 * and store them where they lie, instead of pageable copies through the
 * driver; limbs not 16-byte aligned take the copies.  On by default where
 * supported; yell_set_host_access(0) forces the copies (results are the
 * same).  yell_host_access reports whether the current device uses it. */
int yell_set_host_access(int enable);
int yell_host_access(int* in_use);

/* ---- device-resident calls (device pointers, asynchronous on `stream`) --
 * A batch is `count` polys of L limbs laid out (count, L, N) contiguous;
 * limb l of every poly uses prime cm0 + l. */
int yell_dev_ntt(uint64_t* d_polys, uint32_t count, uint32_t L, uint32_t log_n, uint32_t cm0,
                 int direction, void* stream);
/* Limbs anywhere: d_limbs and d_cms are DEVICE arrays of `count` limb
 * pointers and modulus indices. */
int yell_dev_ntt_limbs(uint64_t* const* d_limbs, const uint32_t* d_cms, uint32_t count,
                       uint32_t log_n, int direction, void* stream);
int yell_dev_elementwise(int op, uint64_t* d_dst, const uint64_t* d_a, const uint64_t* d_b,
                         uint32_t count, uint32_t L, uint32_t log_n, uint32_t cm0, void* stream);
/* Fused polymul of `pairs` pairs; d_c may not alias d_a or d_b.  Degrees
 * with a two-pass polymul (N >= 2^13) need scratch of
 * yell_polymul_scratch_words() words; pass NULL to have the library take it
 * stream-ordered from its per-device memory pool on `stream` and give it back
 * there after the kernels, so the call returns without waiting for the GPU
 * either way.  pairs * L must fit one launch (YELL_ERR_INVALID_ARGUMENT
 * otherwise, in particular for any product >= 2^32); scratch_words() returns
 * 0 for such sizes. */
size_t yell_polymul_scratch_words(uint32_t pairs, uint32_t L, uint32_t log_n);
int yell_dev_polymul(uint64_t* d_c, const uint64_t* d_a, const uint64_t* d_b, uint32_t pairs,
                     uint32_t L, uint32_t log_n, uint32_t cm0, uint64_t* d_scratch,
                     size_t scratch_words, void* stream);
/* ---- batched polymul of uneven sizes (no counterpart in the reference) ----
 * Each entry is one polymul c = a * b of its own degree and limb count: a, b,
 * c are (L, N) device arrays, limb l using prime cm0 + l.  Entries are
 * bucketed by degree; each bucket runs as one launch sequence over all its
 * limbs, buckets run concurrently, and the whole batch is a CUDA graph cached
 * per batch shape (the sequence of (degree, total limbs) buckets), so a batch
 * of a shape seen before costs one list upload and one graph launch.  Outputs
 * of different entries must not overlap.  Asynchronous on `stream`. */
typedef struct yell_polymul_desc {
  uint64_t* c;
  const uint64_t* a;
  const uint64_t* b;
  uint32_t log_n;
  uint32_t L;
  uint32_t cm0;
  uint32_t reserved;
} yell_polymul_desc;
int yell_dev_polymul_batch(const yell_polymul_desc* descs, uint32_t n, void* stream);
/* The same batch as ONE launch of a persistent kernel driven by a device
 * work queue: resident CTAs take work items (whole-limb tiles; for
 * N >= 2^13 the column pass, row step and inverse column pass of each tile)
 * in queue order from a device ticket counter; a step waits for the steps of
 * its limb it depends on.  Each wait is bounded (2 s); one that runs out
 * records YELL_ERR_TIMEOUT, read (and cleared) by yell_batch_queue_status,
 * which waits for the queued work.  Asynchronous on `stream`. */
int yell_dev_polymul_batch_queue(const yell_polymul_desc* descs, uint32_t n, void* stream);
/* The same work items as THREE launches in queue order, one per phase
 * (forward column passes and whole-limb tiles; row steps; inverse column
 * passes), each kernel with its own register budget.  Launch order carries
 * the dependencies, so nothing waits on the device.  Asynchronous on
 * `stream`; results identical to yell_dev_polymul_batch. */
int yell_dev_polymul_batch_phased(const yell_polymul_desc* descs, uint32_t n, void* stream);
int yell_batch_queue_status(uint32_t* status);
/* Check of the bounded wait: a queue whose row steps wait on column passes
 * that are never queued; every wait runs out after timeout_ns (<= 10 s) and
 * *status receives YELL_ERR_TIMEOUT.  Synchronous. */
int yell_batch_queue_wait_check(uint64_t timeout_ns, uint32_t* status);

/* ---- serving loop (no counterpart in the reference) ------------------------
 * Continuous batching of polymul and NTT requests of mixed size.  A scheduler thread
 * owns max_inflight stream slots; whenever one is free it admits queued
 * requests in arrival order while an HBM budget (a device arena allocated at
 * create time) can hold their buffers, and launches everything admitted as
 * one batch, so requests arriving while other batches run overlap with them
 * on the device.  Host-memory requests are copied in and out by the server;
 * YELL_REQ_DEVICE requests use caller-owned device buffers (only scratch, and
 * the output with YELL_REQ_DISCARD_OUTPUT, come from the budget). */
typedef struct yell_server yell_server;
typedef struct yell_server_config {
  uint64_t hbm_budget_bytes;       /* arena size; 0 = 120 GiB capped by free memory */
  uint32_t max_inflight;           /* concurrent batches (stream slots); 0 = 4 */
  uint32_t max_batch;              /* requests per batch; 0 = 1024; 1 = per-call serving */
  uint32_t inject_alloc_failures;  /* test hook: refuse this many admissions (OOM) */
  uint32_t reserved;
} yell_server_config;
enum yell_request_flags {
  YELL_REQ_HOST = 0,            /* a, b, c are host arrays of L*N words */
  YELL_REQ_DEVICE = 1,          /* a, b, c are device arrays (16-byte aligned) */
  YELL_REQ_DISCARD_OUTPUT = 2,  /* compute into a server buffer and drop it (load tests) */
  /* the request's operation (none of these: polymul c = a * b) */
  YELL_REQ_NTT_FORWARD = 4,     /* c = ntt<N>::forward(a), b unused */
  YELL_REQ_NTT_BACKWARD = 8     /* c = ntt<N>::backward(a), b unused */
};
typedef struct yell_polymul_request {
  const uint64_t* a;
  const uint64_t* b;
  uint64_t* c;
  uint32_t log_n;
  uint32_t L;
  uint32_t cm0;
  uint32_t flags;
} yell_polymul_request;
typedef struct yell_request_result {
  int status;
  double queue_us;    /* submit -> admitted */
  double latency_us;  /* submit -> completion observed */
} yell_request_result;
typedef struct yell_server_stats {
  uint64_t submitted, completed, rejected, cancelled, failed, batches, queued;
  uint64_t hbm_budget, hbm_in_use, hbm_peak;
  double p50_us, p99_us, mean_us, max_us;
  double limb_ntts, limb_ntts_per_s, requests_per_s, window_s;
} yell_server_stats;
int yell_server_create(const yell_server_config* cfg, yell_server** out);
int yell_server_destroy(yell_server* s);
/* Validates and queues; YELL_ERR_BUDGET if the request can never fit. */
int yell_server_submit(yell_server* s, const yell_polymul_request* r, uint64_t* id);
/* Bounded wait: YELL_ERR_TIMEOUT after timeout_s; the request's own status otherwise. */
int yell_server_wait(yell_server* s, uint64_t id, double timeout_s, yell_request_result* out);
/* Cancels a request that has not been admitted yet. */
int yell_server_cancel(yell_server* s, uint64_t id);
/* Holds (1) or releases (0) admission; queued requests stay queued. */
int yell_server_pause(yell_server* s, int paused);
int yell_server_get_stats(yell_server* s, int reset, yell_server_stats* out);
/* Poisson arrivals at offered_rps for duration_s drawn round-robin from the
 * templates (outputs discarded), then a bounded drain; fills `out`. */
int yell_server_load_test(yell_server* s, const yell_polymul_request* templates, uint32_t n,
                          double offered_rps, double duration_s, uint64_t seed, yell_server_stats* out);

/* ---- 32-bit moduli mode: the reference built with -DYELL_USE_32BITS_MODULI
 * (include/yell/params.hpp:2-6, params_32.hpp:15-34): 291 30-bit primes
 * p = 1 mod 2^16, uint32 words, uint64 products, N = 2^3 .. 2^15.  Same call
 * meanings as the 64-bit functions above with uint32_t words; modulus
 * indices address the 32-bit prime table. ---------------------------------- */
uint32_t yell32_max_moduli(void);      /* kMaxNbModuli = 291 */
uint32_t yell32_max_log_degree(void);  /* log2 kMaxPolyDegree = 15 */
uint32_t yell32_prime(uint32_t cm);          /* params::P[cm] */
uint32_t yell32_prime_pn(uint32_t cm);       /* params::Pn[cm] */
uint32_t yell32_primitive_root(uint32_t cm); /* params::primitive_roots[cm], order 2^16 */
int yell32_ntt_tables(uint32_t log_n, uint32_t cm, uint32_t* out4n, uint32_t* scalars4);
int yell32_init_ntt_tables(uint32_t log_n, uint32_t cm0, uint32_t L);
/* ntt<N>::forward / forward_lazy / backward (include/yell/ntt.hpp:59-65) */
int yell32_ntt_forward(uint32_t* op, uint32_t log_n, uint32_t cm);
int yell32_ntt_forward_lazy(uint32_t* op, uint32_t log_n, uint32_t cm);
int yell32_ntt_backward(uint32_t* op, uint32_t log_n, uint32_t cm);
/* device batches laid out (count, L, N) uint32, 16-byte aligned */
int yell32_dev_ntt(uint32_t* d_polys, uint32_t count, uint32_t L, uint32_t log_n, uint32_t cm0,
                   int direction, void* stream);
int yell32_dev_polymul(uint32_t* d_c, const uint32_t* d_a, const uint32_t* d_b, uint32_t pairs,
                       uint32_t L, uint32_t log_n, uint32_t cm0, void* stream);
/* At N = 2^14 and 2^15 the polymul's CTAs wait on the device for the bulk
 * copies that bring their operands into shared memory, each wait for at most
 * 1 s.  A wait that runs out records YELL_ERR_TIMEOUT and the kernel still
 * finishes (its output is then undefined).  This call waits for all work
 * queued on the current device, stores the recorded status (YELL_OK or
 * YELL_ERR_TIMEOUT) in *status and clears it.  No counterpart in the
 * reference, whose calls do not wait on a device. */
int yell32_wait_status(uint32_t* status);
/* Check of that bounded wait: a one-CTA kernel announces copies on an
 * mbarrier, starts none, and waits as the polymul kernels do; the wait runs
 * out after timeout_ns (<= 10 s) and *status receives YELL_ERR_TIMEOUT (read
 * and cleared as by yell32_wait_status).  Synchronous. */
int yell32_wait_check(uint64_t timeout_ns, uint32_t* status);
int yell32_dev_elementwise(int op, uint32_t* d_dst, const uint32_t* d_a, const uint32_t* d_b,
                           uint32_t count, uint32_t L, uint32_t log_n, uint32_t cm0, void* stream);
/* poly<N> members on host limbs (moduli 0 .. L-1), as yell_poly_* above */
int yell32_poly_forward(uint32_t* const* limbs, uint32_t L, uint32_t log_n);
int yell32_poly_forward_lazy(uint32_t* const* limbs, uint32_t L, uint32_t log_n);
int yell32_poly_backward(uint32_t* const* limbs, uint32_t L, uint32_t log_n);
int yell32_poly_mulmod(uint32_t* const* dst, const uint32_t* const* a, const uint32_t* const* b, uint32_t L,
                       uint32_t log_n);
int yell32_poly_addmod(uint32_t* const* dst, const uint32_t* const* a, const uint32_t* const* b, uint32_t L,
                       uint32_t log_n);
int yell32_poly_submod(uint32_t* const* dst, const uint32_t* const* a, const uint32_t* const* b, uint32_t L,
                       uint32_t log_n);
int yell32_poly_add_product_of(uint32_t* const* acc, const uint32_t* const* a, const uint32_t* const* b,
                               uint32_t L, uint32_t log_n);
int yell32_poly_negate(uint32_t* const* limbs, uint32_t L, uint32_t log_n);

/* ---- device-resident poly handles (the device-side poly<N>) -------------
 * A handle owns one poly in HBM: L limbs of N words, limb l under prime
 * cm0 + l (the reference's poly<N>(nmoduli) uses cm0 = 0;
 * include/yell/poly.hpp:43-121).  upload / download take L host limb
 * pointers like raw_data() and are synchronous; every other call is ordered
 * on the device's library stream.  Handles in one call must agree in N, L and
 * cm0. */
typedef struct yell_dev_poly yell_dev_poly;
int yell_dev_poly_alloc(uint32_t L, uint32_t log_n, uint32_t cm0, yell_dev_poly** out);
int yell_dev_poly_free(yell_dev_poly* p);
int yell_dev_poly_info(const yell_dev_poly* p, uint64_t** d_data, uint32_t* L, uint32_t* log_n, uint32_t* cm0);
int yell_dev_poly_upload(yell_dev_poly* p, const uint64_t* const* limbs);
int yell_dev_poly_download(const yell_dev_poly* p, uint64_t* const* limbs);
/* poly<N>::forward / forward_lazy / backward (details/poly.hpp:170-186) */
int yell_dev_poly_ntt(yell_dev_poly* p, int direction);
/* dst = a op b with op a yell_elementwise_op: operator* + - and their
 * assigning forms (dst may be a), add_product_of (MULADD), negate (b NULL) */
int yell_dev_poly_op(int op, yell_dev_poly* dst, const yell_dev_poly* a, const yell_dev_poly* b);
/* c = a * b in Z_Q[X]/(X^N + 1): forward, mulmod, backward fused; c is not a or b */
int yell_dev_poly_mul(yell_dev_poly* c, const yell_dev_poly* a, const yell_dev_poly* b);
/* Asynchronous batch of n products c[i] = a[i] * b[i] of any mix of sizes
 * (run as yell_dev_polymul_batch); the ticket completes with the batch.
 * yell_batch_wait returns YELL_ERR_TIMEOUT after timeout_s (the ticket stays
 * valid) and frees the ticket otherwise; yell_batch_release drops a ticket
 * without waiting. */
typedef struct yell_batch yell_batch;
int yell_batch_submit(yell_dev_poly* const* c, const yell_dev_poly* const* a, const yell_dev_poly* const* b,
                      uint32_t n, yell_batch** ticket);
int yell_batch_wait(yell_batch* t, double timeout_s);
int yell_batch_release(yell_batch* t);

/* ---- seeded device samplers: replace poly<N>::set(uniform / ZO_dist / hwt_dist /
 * gaussian) (include/yell/details/poly.hpp:195-330) -------------------------
 * Fill `count` polys (count, L, N) on the device.  The reference's samplers
 * draw bytes from an unseeded stream (yell::fastrandombytes); these draw from
 * a seeded one, word k = splitmix64(seed + (k + 1) * 0x9E3779B97F4A7C15),
 * bytes little-endian, and make of it exactly what the reference's set(...)
 * makes of the same stream: uniform (one word per coefficient, limb after
 * limb, poly after poly: mask to 2^(floor(log2 p)+1) then subtract p once),
 * ZO (one byte r per coefficient, poly after poly: r <= rho ? (r & 2 ? -1 : 1)
 * : 0), HWT (poly j on the stream seeded with word j of this seed's stream:
 * the reference's reservoir sampling with rejection, sorted positions signed
 * +-1 by the words after the draws).  gaussian: a centred integer |e| <= tail
 * by inversion of word k against the cumulative table of
 * yell_gaussian_table, times `amplifier` as in the reference's
 * gaussian{prng, amp} (tail <= 1024, tail*amplifier < 2^61); its distribution
 * is the reference's FastGaussianNoise's to within 2^-63 per value, its draws
 * are not.  ZO, HWT and gaussian coefficients are the same integers in every
 * limb, mapped e < 0 ? p + e : e.  HWT takes scratch stream-ordered from the
 * library's per-device pool. */
int yell_dev_sample_uniform(uint64_t* d_out, uint32_t count, uint32_t L, uint32_t log_n, uint32_t cm0,
                            uint64_t seed, void* stream);
int yell_dev_sample_zo(uint64_t* d_out, uint32_t count, uint32_t L, uint32_t log_n, uint32_t cm0,
                       uint32_t rho, uint64_t seed, void* stream);
int yell_dev_sample_hwt(uint64_t* d_out, uint32_t count, uint32_t L, uint32_t log_n, uint32_t cm0,
                        uint32_t h, uint64_t seed, void* stream);
int yell_dev_sample_gaussian(uint64_t* d_out, uint32_t count, uint32_t L, uint32_t log_n, uint32_t cm0,
                             double sigma, uint32_t tail, uint64_t amplifier, uint64_t seed, void* stream);
/* The cumulative table of yell_dev_sample_gaussian for (sigma, tail) on the
 * host: out[i] = floor(2^64 * P(e <= i - tail)) for i < 2 * tail, out[2 * tail]
 * = 2^64 - 1 (cap >= 2 * tail + 1).  It stands in for the barrier table the
 * reference's FastGaussianNoise builds with MPFR
 * (include/yell/prng/FastGaussianNoise.hpp:302-374). */
int yell_gaussian_table(double sigma, uint32_t tail, uint64_t* out, uint32_t cap);

/* ---- RNS -> big-integer lifting: replaces gmp::poly2mpz
 * (include/yell/gmp.hpp:42-70, tables lib/gmp.cpp:6-51) ----------------------
 * Coefficient i of a poly with residues r_j mod q_j (moduli cm0 .. cm0+L-1,
 * L <= 400) lifts to the unique x in [0, Q), Q = prod q_j, x = r_j mod q_j:
 * the value poly2mpz returns for residues below their moduli (the form
 * backward() leaves).  x is written as W little-endian 64-bit words
 * (W = yell_crt_words(L, cm0); mpz_import(z, W, -1, 8, 0, 0, words) makes the
 * mpz_t), coefficient-major: words [i*W, (i+1)*W) of the output. */
int yell_crt_words(uint32_t L, uint32_t cm0, uint32_t* words);
/* d_in: count polys (count, L, N); d_out: count * N * W words. */
int yell_dev_crt_lift(uint64_t* d_out, const uint64_t* d_in, uint32_t count, uint32_t L, uint32_t log_n,
                      uint32_t cm0, void* stream);
/* Host drop-in for poly2mpz over moduli 0 .. L-1: limbs[j] -> out (N * W words). */
int yell_poly_to_bigint(uint64_t* out, const uint64_t* const* limbs, uint32_t L, uint32_t log_n);

/* ---- launch variants and the autotuner (no counterpart in the reference) --
 * Every degree has one or more launch variants that apply exactly the same
 * butterflies (same output words) with a different split of the work: limbs
 * per CTA for whole-limb degrees, column/row split k1 for 2^13 and up
 * (2^13 has both kinds).
 * yell_autotune times the fused polymul of every variant of log_n on
 * synthetic data of the given size on the current device and selects the
 * fastest; with YELL_GB300_TUNE_FILE set the choice is saved there and
 * reloaded when the library first uses the device. */
int yell_variant_count(uint32_t log_n, uint32_t* count);
int yell_variant_name(uint32_t log_n, uint32_t variant, char* buf, size_t len);
int yell_set_variant(uint32_t log_n, uint32_t variant);
int yell_get_variant(uint32_t log_n, uint32_t* variant);
int yell_autotune(uint32_t log_n, uint32_t L, uint32_t pairs, uint32_t* best, double* best_ms);

/* Integer roofline (no counterpart in the reference): runs the production CT
 * and GS butterflies on register-resident words with no memory traffic on
 * every SM of the current device and returns butterflies per second, the
 * ceiling the 64-bit modular arithmetic allows at the current clock. */
int yell_calibrate_butterflies(double* ct_per_s, double* gs_per_s);
/* The same for the 32-bit moduli mode's butterflies on 32-bit words. */
int yell32_calibrate_butterflies(double* ct_per_s, double* gs_per_s);

/* Waits for all work the library queued on its own stream of this device. */
int yell_synchronize(void);

/* Fused polymul that allocates nothing (no counterpart in the reference).
 * For callers that cannot allocate device memory: a process whose HBM is
 * owned by a fixed budget or a pooled allocator that forbids allocations
 * outside the pool, or a latency-critical caller that cannot afford
 * cudaMalloc/cudaFree synchronising the device.  Same arguments and results
 * as yell_dev_polymul, but the scratch of the two-pass degrees (2^13 and up)
 * is a fixed 16 MiB device array inside the library (2^21 words: at most
 * 2^21 / N limbs = pairs * L per call, e.g. 32 limbs at N = 2^16); larger
 * calls return YELL_ERR_INVALID_ARGUMENT, except at 2^13, where they run the
 * whole-limb polymul, which needs no scratch.  The twiddle tables must already be
 * resident (yell_init_ntt_tables_range), since building them allocates; the
 * first table build on a device also brings the array up and looks up its
 * device address, so the array's memory is taken then and no call of this
 * function allocates or does set-up.  All calls share the one array: calls
 * whose GPU work overlaps (other streams, other host threads) race on it, so
 * order them on one stream.  The array needs no clearing: each call writes
 * the scratch it reads. */
int yell_dev_polymul_noalloc(uint64_t* d_c, const uint64_t* d_a, const uint64_t* d_b,
                             uint32_t pairs, uint32_t L, uint32_t log_n, uint32_t cm0,
                             void* stream);

/* ---- launch profiling (no counterpart in the reference) -----------------
 * Between start and stop every kernel the library launches is bracketed by
 * CUDA events on its stream; stop waits for them and totals the device time
 * per kernel name.  get() returns the i-th kernel's name, launch count and
 * total milliseconds. */
int yell_profile_start(void);
int yell_profile_stop(void);
int yell_profile_count(void);
int yell_profile_get(int i, char* name, size_t name_len, uint64_t* launches, double* total_ms);

#ifdef __cplusplus
}
#endif

#endif /* YELL_GB300_H_ */
