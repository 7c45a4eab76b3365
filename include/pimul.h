/*
 * pimul — GB300-native big-integer multiply engine (C ABI).
 *
 * Numbers are little-endian arrays of 64-bit limbs, as in the reference's
 * `Integer` magnitude (joelodom/pi crates/bignum/src/integer.rs:22-27).  An
 * empty array (length 0) is zero.  Products are exact: every result equals
 * the reference's CPU multiply bit for bit.
 *
 * The multiply is a Goldilocks-prime (p = 2^64 - 2^32 + 1) number-theoretic
 * transform with the reference's own rules: 16-bit coefficients, four per
 * limb, transform length N = next_pow2(4*la + 4*lb - 1)
 * (crates/bignum/src/ntt.rs:633-634, ntt.rs:810-813), N <= 2^32.
 *
 * Every entry point returns PIMUL_OK (0) or one of the error codes below;
 * pimul_last_error() gives a message for the calling thread's last failure.
 * All entry points are thread-safe and re-entrant.
 */
#ifndef PIMUL_H
#define PIMUL_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PIMUL_OK 0
#define PIMUL_EINVAL 1     /* bad argument (null pointer, capacity too small, N > 2^32) */
#define PIMUL_ENOMEM 2     /* device allocation failed or HBM budget exceeded */
#define PIMUL_ECUDA 3      /* a CUDA call failed */
#define PIMUL_ETIMEDOUT 4  /* a bounded wait ran out */
#define PIMUL_ENOTFOUND 5  /* unknown handle or ticket */
#define PIMUL_ECANCELED 6  /* request was cancelled */

/* Library version string. */
const char* pimul_version(void);

/* Message for the calling thread's last failed call ("" if none). */
const char* pimul_last_error(void);

/* Select and initialise the CUDA device (twiddle tables, pools).  Optional:
 * every other entry point initialises device 0 on first use.  Idempotent. */
int pimul_init(int device);

/* Release pooled device memory and tables.  Later calls re-initialise. */
int pimul_shutdown(void);

/*
 * Plain drop-in multiply with HOST buffers: out = a * b, trimmed of top zero
 * limbs; *out_len receives the trimmed length.  out_cap must be >= la + lb
 * (or 0 when la == 0 or lb == 0).  a == b with la == lb takes the squaring
 * path (two transforms instead of three); the bits are the same.
 *
 * Replaces: crates/bignum/src/ntt.rs:806 `mul_mag_ntt(a: &[u64], b: &[u64])
 * -> Vec<u64>`, called from mul_mag_dispatch at crates/bignum/src/integer.rs:480.
 */
int pimul_mul(const uint64_t* a, size_t la, const uint64_t* b, size_t lb,
              uint64_t* out, size_t out_cap, size_t* out_len);

/*
 * Same multiply on DEVICE buffers, asynchronous on `stream` (a cudaStream_t;
 * NULL = the calling thread's own stream).  Writes exactly la + lb limbs to
 * d_out (the top limb may be zero); d_out must not overlap the inputs.
 * la == 0 or lb == 0 is a zero product: nothing is written.
 * Scratch comes from the engine's device pool.
 *
 * Replaces: crates/bignum/src/ntt.rs:806 `mul_mag_ntt`, for callers whose
 * operands already live in HBM.
 */
int pimul_mul_device(const uint64_t* d_a, size_t la, const uint64_t* d_b, size_t lb,
                     uint64_t* d_out, void* stream);

/*
 * The same device multiply for callers that cannot allocate device memory
 * when they multiply (a GPU whose memory belongs to another allocator, a
 * loop where cudaMalloc's implicit synchronisation is not allowed, a runtime
 * that allocates only at start-up).  It uses no memory pool: its scratch is
 * a fixed device array inside this library (17 MiB of scratch plus 18 MiB
 * of root tables, resident on every GPU that loads the library until exit), so products are limited to
 * la + lb <= 262144 limbs (transform length <= 2^20); larger ones return
 * PIMUL_EINVAL.  All calls share that array: calls that overlap on the GPU
 * race and must be serialised by the caller.  The first call on a device
 * sets the array up (address lookup and a synchronous table copy), so make
 * it before any stream capture.  `stream` NULL means the CUDA default stream.
 *
 * No counterpart in the reference (its multiply allocates per call:
 * crates/bignum/src/ntt.rs:823-824 acquires pooled heap buffers).
 */
int pimul_mul_device_noalloc(const uint64_t* d_a, size_t la, const uint64_t* d_b, size_t lb,
                             uint64_t* d_out, void* stream);

/* One product of a batch: device pointers; out receives la + lb limbs. */
typedef struct pimul_job {
  const uint64_t* a;
  size_t la;
  const uint64_t* b;
  size_t lb;
  uint64_t* out;
} pimul_job;

/*
 * Batched form: n independent products on device buffers in one call
 * (asynchronous on `stream`, NULL = the calling thread's stream).  Products
 * are grouped by transform length: up to 2^12 one CTA per product in a
 * persistent kernel, longer ones one launch per pass for the whole group;
 * products of one length whose operand b is the same array (same pointer
 * and length) compute b's transform once.  Each out[i] is written exactly
 * as pimul_mul_device would write it.
 *
 * Replaces: the independent mul_mag calls of one binary-splitting level
 * (crates/pi-core/src/algorithm/chudnovsky.rs:399-413, run through
 * rayon::join), each of which reaches crates/bignum/src/ntt.rs:806.
 */
int pimul_mul_batch(const pimul_job* jobs, size_t n, void* stream);

/*
 * Batched add/subtract of device limb arrays: out[0..nout) = x + y
 * (sub == 0) or x - y (sub != 0, x >= y), operands zero-extended to nout
 * (nout >= max(nx, ny); for an addition max(nx, ny) + 1 holds every carry).
 * Synchronous; PIMUL_EINVAL if a carry or borrow leaves the top limb.
 * sub == PIMUL_SUB_MOD: x - y modulo 2^(64 nout), no borrow check (the low
 * limbs of a difference known to fit in nout limbs); a call whose jobs are
 * all PIMUL_SUB_MOD is asynchronous on `stream`.  out may equal x.
 * Replaces: crates/bignum/src/integer.rs:351-421 (add_mag / sub_mag under
 * Integer addition) for the T sums of a binary-splitting level.
 */
typedef struct pimul_addsub_job {
  const uint64_t* x;
  size_t nx;
  const uint64_t* y;
  size_t ny;
  uint64_t* out;
  size_t nout;
  int sub;
} pimul_addsub_job;
#define PIMUL_SUB_MOD 2
int pimul_addsub_batch(const pimul_addsub_job* jobs, size_t n, void* stream);

/*
 * Sums of two products for many operand sets at once (device pointers):
 * out[0..nout) = a1 b1 + a2 b2, nout >= max(la1 + lb1, la2 + lb2) + 1
 * (limbs above the sum are zeroed; an empty pair, la or lb zero, adds
 * nothing, so a job with one pair is a plain product and nout >= la + lb
 * suffices).  Long sums are added in the transform domain: four forward
 * transforms, one inverse and one carry pass instead of two of each and an
 * addition.  In this call and in pimul_mul_batch, products of one transform
 * length whose operand b is the same array (same pointer and length) share
 * b's transform.  Asynchronous on `stream`.
 * This engine's own addition: the T = T_L Q_R + P_L T_R step of a binary
 * splitting level (crates/pi-core/src/algorithm/chudnovsky.rs:399-413) as
 * one job.
 */
typedef struct pimul_sum_job {
  const uint64_t* a1;
  size_t la1;
  const uint64_t* b1;
  size_t lb1;
  const uint64_t* a2;
  size_t la2;
  const uint64_t* b2;
  size_t lb2;
  uint64_t* out;
  size_t nout;
} pimul_sum_job;
int pimul_sum_batch(const pimul_sum_job* jobs, size_t n, void* stream);

/*
 * pimul_sum_batch with options.  PIMUL_BATCH_WRAP: a job of 2^20 points or
 * more whose coefficients fill at most 5/8 of its transform (and whose
 * operands each fit half of it) runs as a cyclic product of half the length:
 * its top coefficients (at most 2^(L-3) of them) wrap onto the bottom ones
 * and are separated again with the exact low coefficients, from a short
 * product of the operands' low limbs computed first.  Same results as
 * pimul_sum_batch, about half the work for such jobs (the top levels of a
 * 10^9-digit splitting tree run at 51-54 % fill).  Used by the batched pi
 * drivers; the plain drop-in keeps the reference's transform length.
 * This engine's own option; no counterpart in the reference (its
 * mul_mag_ntt, crates/bignum/src/ntt.rs:810-813, always takes the next
 * power of two).
 */
#define PIMUL_BATCH_WRAP 1u
int pimul_sum_batch_ex(const pimul_sum_job* jobs, size_t n, void* stream, unsigned flags);

/* Trimmed lengths (highest nonzero limb + 1) of n device limb arrays of
 * lengths lens[i]; out_lens on the host.  Synchronous. */
int pimul_top_limbs(const uint64_t* const* arrays, const size_t* lens, size_t n, size_t* out_lens, void* stream);

/*
 * Batch plans: a fixed batch shape (la[i], lb[i]) laid out once, with all its
 * launches captured into a CUDA graph.  plan_run takes jobs of exactly that
 * shape (new pointers each time) and replays the graph; runs of one plan are
 * serialised (a run waits until the previous run has read its descriptors).
 * This engine's own addition (the per-level schedule of a product tree).
 */
typedef struct pimul_batch_plan pimul_batch_plan;
int pimul_batch_plan_create(const size_t* la, const size_t* lb, size_t n, pimul_batch_plan** plan);
int pimul_batch_plan_run(pimul_batch_plan* plan, const pimul_job* jobs, size_t n, void* stream);
int pimul_batch_plan_destroy(pimul_batch_plan* plan);

/*
 * Autotuner: times the candidate pass counts per transform for every
 * transform length 2^log_n_min .. 2^log_n_max on `reps` synthetic products
 * (each count split into radices 2^6 .. 2^9, the first at least 2^7, with
 * the fewest radix-8/4 rounds), and the one-CTA kernel's persistent grid
 * (CTAs per SM); keeps the fastest for later calls and writes a JSON
 * report.  pimul_tuning_set applies saved choices (passes = 0: default
 * count, ceil(log_n / 9) and at least 2; ctas <= 0: unchanged).
 * The transform length itself is the reference's rule and is not tuned.
 */
int pimul_autotune(int log_n_min, int log_n_max, int reps, char* report, size_t report_cap);
int pimul_tuning_set(int log_n, int passes, int small_ctas_per_sm);

/*
 * Twiddle-table cache.  The first and middle passes of a transform read
 * their twiddles from tables laid out like the data (one coalesced load per
 * element; the inverse first pass's table also carries the 1/N scaling),
 * built on first use per transform shape and kept until pimul_shutdown.
 * First passes use tables up to transform length 2^28 (8 N bytes per
 * direction); longer transforms, and shapes past the cap, compute their
 * twiddles.  pimul_twiddle_cache sets the cap in bytes (default 8 GiB;
 * 0: build no more tables) for tables built from then on and reports the
 * bytes already held in *held (may be NULL).  The cache is device memory
 * outside the served form's HBM budget.
 *
 * Replaces: the twiddle cache of crates/bignum/src/ntt.rs:571-611 (the
 * reference caches its per-length twiddles up to a 2^28 cap too).
 */
int pimul_twiddle_cache(uint64_t max_bytes, uint64_t* held);

/*
 * Served form: a device-resident multiply service.
 *
 * Integers live on the device as handles.  pimul_submit queues a product
 * (op PIMUL_OP_MUL: a * b; PIMUL_OP_SQR: a * a), a sum (PIMUL_OP_ADD:
 * a + b, stored in max(la, lb) + 1 limbs) or a difference (PIMUL_OP_SUB:
 * a - b for values a >= b, stored in max(la, lb) limbs; a smaller a gives
 * the difference modulo 2^(64 max(la, lb))) and returns its result
 * handle and a ticket at once; the result handle may be an input of later
 * submits before it is computed (the dependency is a CUDA event: no host
 * round trip).  A service thread admits queued requests whose inputs are
 * launched, in order, while their result and scratch memory fit the HBM
 * budget (pimul_set_budget,
 * default 120 GiB; handles count against it until freed), launches each
 * admitted group as one batch, and releases the scratch when the group
 * completes; requests that arrive meanwhile join the next group (continuous
 * batching).  Groups run on four streams (products and sums in separate
 * groups); a request with a transform of 2^24 or more (pimul_service_config)
 * forms its own group on a high-priority stream.  pimul_wait blocks until a
 * ticket's result is done (timeout_us < 0: no limit) or returns
 * PIMUL_ETIMEDOUT.  pimul_free waits for the handle's producer and readers;
 * pimul_release returns at once and the handle is freed when they are done
 * (a tree of chained requests releases its inner nodes this way).
 * pimul_adopt makes a handle of device memory the caller owns and keeps
 * (never freed by the service, not counted in the budget); pimul_handle_device
 * waits for a handle's producer and gives its device address and stored
 * length.  A product handle stores la + lb limbs; pimul_download returns the
 * trimmed value.
 * pimul_service_stats reports submit-to-completion latency percentiles.
 *
 * Replaces: the per-level products of the binary-splitting tree with their
 * operands kept in HBM between levels (crates/pi-core/src/algorithm/
 * chudnovsky.rs:377-413, where each Integer * Integer reaches
 * crates/bignum/src/ntt.rs:806 through crates/bignum/src/integer.rs:637).
 */
#define PIMUL_OP_MUL 0
#define PIMUL_OP_SQR 1
#define PIMUL_OP_ADD 2
#define PIMUL_OP_SUB 3
int pimul_set_budget(uint64_t bytes);
int pimul_upload(const uint64_t* host, size_t n, uint64_t* handle);
int pimul_submit(int op, uint64_t a, uint64_t b, uint64_t* out_handle, uint64_t* ticket);
int pimul_wait(uint64_t ticket, int64_t timeout_us);
int pimul_handle_size(uint64_t handle, size_t* limbs);
int pimul_download(uint64_t handle, uint64_t* host, size_t cap, size_t* len);
int pimul_free(uint64_t handle);
int pimul_release(uint64_t handle);
int pimul_adopt(const uint64_t* d, size_t n, uint64_t* handle);
int pimul_handle_device(uint64_t handle, const uint64_t** d, size_t* limbs);
int pimul_service_stats(double* p50_ms, double* p99_ms, uint64_t* completed, uint64_t* batches,
                        uint64_t* bytes_in_use);
int pimul_service_reset_stats(void);

/* Admission policy of the service: requests whose transform length is
 * 2^big_log_n or more run alone on the high-priority stream (default 24),
 * smaller ones are grouped, at most max_batch per group (default 4096);
 * values <= 0 leave a setting unchanged.  No counterpart in the reference
 * (it has no multiply service). */
int pimul_service_config(int big_log_n, int max_batch);

/* pimul_mul's contract (host buffers, trimmed result, squares when a == b)
 * carried out through the served form: upload, submit, wait, download,
 * free.  Same signature as pimul_mul, so it can be a pimul_mul_fn backend. */
int pimul_mul_served(const uint64_t* a, size_t la, const uint64_t* b, size_t lb, uint64_t* out, size_t out_cap,
                     size_t* out_len);

/* Signature of a multiply backend: pimul_mul's own. */
typedef int (*pimul_mul_fn)(const uint64_t* a, size_t la, const uint64_t* b, size_t lb, uint64_t* out,
                            size_t out_cap, size_t* out_len);

/*
 * Digits of pi by Chudnovsky binary splitting, driven from the host with
 * every product at or above the NTT threshold (ntt_threshold limbs of the
 * smaller operand; 0 = the reference's 8192) sent to `backend`
 * (NULL = pimul_mul, the GPU engine; one call per product).  Writes
 * `digits` characters "31415..." (no decimal point) to out.  Optional
 * outputs: phase_ms[3] = binary splitting, final assembly, decimal
 * conversion wall times; ntt_products = number of backend calls;
 * ntt_hist33[L] = backend calls with transform length 2^L.
 *
 * Re-entrant: the backend, the threshold, the error state and the
 * statistics belong to the call (the pi drivers below and pimul_to_decimal
 * alike), so calls from different host threads may run at the same time.
 * The first backend error stops the run: no later product is issued, and
 * the call returns that backend's code.
 *
 * Replaces: crates/pi-core/src/algorithm/chudnovsky.rs:75 Chudnovsky::compute
 * with crates/pi-core/src/algorithm/util.rs:25 write_decimal_digits, whose
 * multiplies all reach crates/bignum/src/ntt.rs:806 through
 * crates/bignum/src/integer.rs:445.
 */
int pimul_pi_chudnovsky(uint64_t digits, char* out, size_t cap, pimul_mul_fn backend, uint64_t ntt_threshold,
                        double* phase_ms, uint64_t* ntt_products, uint64_t* ntt_hist33);

/*
 * Batched, device-resident form of pimul_pi_chudnovsky.  The binary
 * splitting runs level by level: leaves of leaf_terms terms (0: chosen per
 * eighth of the terms, at most 64, so that each level's products fill
 * their transform lengths; at most 64 in any case) are computed on the
 * device;
 * the lowest levels (every node pair's products within 2^12 points) merge
 * one pair per thread group in shared memory (P, Q and the fused T sum from
 * six forward and three inverse transforms), with the levels' schedule
 * captured as one CUDA graph per segment and the trimmed lengths kept on
 * the device; every level above keeps P, Q and T in HBM, with all of the
 * level's products in one pimul_sum_batch call (Q_L Q_R, P_L P_R, and
 * T_L Q_R + P_L T_R as one fused sum; Q_L Q_R and T_L Q_R share Q_R's
 * transform) and the trimmed lengths from pimul_top_limbs.  Environment:
 * PIMUL_PI_MERGED_LEVELS=0 runs the lowest levels through pimul_sum_batch
 * too, PIMUL_PI_LEVEL_GRAPH=0 launches the merged levels one by one instead
 * of through the graph (same kernels; for profilers).  The root's Q and T stay in HBM
 * for the final assembly (a Newton reciprocal of A Q + T on the device) and
 * the decimal conversion (level-batched with its nodes in HBM, as
 * pimul_to_decimal); only the digits return to the host.  The conversion's
 * divisors and reciprocals, sqrt(10005) (by a multiplication-only Newton
 * iteration) and the decimal scale are computed beside the splitting.
 * Optional outputs: phase_ms[3] as above; gpu_products = products sent to
 * the GPU (batched and plain); levels = batched splitting levels;
 * ntt_hist33[L] = products with transform 2^L.  The digits are identical to
 * pimul_pi_chudnovsky's.
 *
 * Replaces: crates/pi-core/src/algorithm/chudnovsky.rs:75 Chudnovsky::compute,
 * whose binary splitting (chudnovsky.rs:377-413) issues each level's
 * products as independent rayon tasks.
 */
int pimul_pi_chudnovsky_batched(uint64_t digits, char* out, size_t cap, uint64_t leaf_terms, double* phase_ms,
                                uint64_t* gpu_products, uint64_t* levels, uint64_t* ntt_hist33);

/*
 * pimul_pi_chudnovsky_batched with the splitting tree's upper levels driven
 * through the multiply service: the level-batched device splitting stops at
 * about serve_nodes nodes (0: 512), which become handles (pimul_adopt), and
 * the rest of the tree is submitted as the recursion unfolds, five chained
 * requests per merge (the three products, the T cross products' sum or
 * difference), inner nodes released as their parents are queued; only the
 * root's Q and |T| are read, by the device final assembly.  Same digits.
 * Optional outputs as pimul_pi_chudnovsky_batched; requests = service
 * requests submitted.
 *
 * Replaces: the binary splitting's recursion of
 * crates/pi-core/src/algorithm/chudnovsky.rs:377-413, whose products and
 * sums of one level run as independent rayon tasks.
 */
int pimul_pi_chudnovsky_served(uint64_t digits, char* out, size_t cap, uint64_t serve_nodes, double* phase_ms,
                               uint64_t* gpu_products, uint64_t* requests);

/*
 * Decimal string of the non-negative integer limbs[0..n) (little-endian u64,
 * "0" for n == 0 or zero), without a terminator.  *len receives the length;
 * a NULL or short `out` returns PIMUL_EINVAL after setting *len.  batched = 0:
 * the reference's recursive divide and conquer (large products one GPU call
 * each); batched != 0: level by level on powers 10^(19 2^k) with each
 * level's products in one pimul_mul_batch call.  Both give the same string.
 *
 * Replaces: crates/bignum/src/integer.rs:892 Integer::to_string (the divide
 * and conquer of integer.rs:892-983).
 */
int pimul_to_decimal(const uint64_t* limbs, size_t n, char* out, size_t cap, size_t* len, int batched);

/*
 * verify-hex's decimal -> hex conversion of pi: text[0..len) is "3." and E
 * decimal digits (ASCII whitespace around it is ignored); out receives "3."
 * and the h = floor(E log2(10) / 4) hex digits (lower case) of
 * m = floor(N 16^h / 10^E) after its leading 3, N the E + 1 digits as an
 * integer, without a terminator or newline.  *out_len = h + 2 is set before
 * `out` and `cap` are checked (a NULL or short out returns PIMUL_EINVAL).
 * PIMUL_EINVAL with the reference's messages for text not starting with
 * "3.", non-digit characters or E > 2^32 - 1.  Parsing, 10^E, the quotient
 * and the hex digits all run on the device (parse: 19-digit chunks, then
 * x = hi 10^(19 2^k) + lo level by level through pimul_mul_batch; quotient:
 * a Newton reciprocal and an exact remainder correction).  phase_ms
 * (optional, 4 entries): parse, power of ten, quotient, hex digits.
 *
 * Replaces: crates/pi-cli/src/verify_hex.rs:553-629 convert_decimal_to_hex
 * (its quadratic Integer::parse_radix, integer.rs:102-153, and the
 * division of integer.rs:1004-1083) up to writing the file.
 */
int pimul_decimal_to_hex(const char* text, size_t len, char* out, size_t cap, size_t* out_len, double* phase_ms);

/*
 * Digits of pi by the Gauss-Legendre AGM, same conventions as
 * pimul_pi_chudnovsky (phase_ms: iterations + final assembly, unused,
 * decimal conversion).
 *
 * Replaces: crates/pi-core/src/algorithm/gauss_legendre.rs:61
 * GaussLegendre::compute with util.rs:25 write_decimal_digits.
 */
int pimul_pi_gauss_legendre(uint64_t digits, char* out, size_t cap, pimul_mul_fn backend, uint64_t ntt_threshold,
                            double* phase_ms, uint64_t* ntt_products);

/* pimul_pi_gauss_legendre with options: PIMUL_PI_FAST_SQRT takes the square
 * roots by a multiplication-only Newton iteration for 1/sqrt(x) instead of
 * the reference's division-based one (float.rs:85-174);
 * PIMUL_PI_DEVICE_DECIMAL converts to decimal with the nodes on the device
 * (the level-batched conversion of pimul_to_decimal) instead of the
 * reference's recursion (util.rs:25-83).  The digits are the same. */
#define PIMUL_PI_FAST_SQRT 1u
#define PIMUL_PI_DEVICE_DECIMAL 2u
/* PIMUL_PI_DEVICE_AGM: the whole iteration on the device in fixed point
 * (a, b, t in HBM, square roots by a Newton iteration for 1/sqrt(x) carried
 * from step to step), then the device quotient and decimal conversion; the
 * backend is not used.  The digits are the same. */
#define PIMUL_PI_DEVICE_AGM 4u
int pimul_pi_gauss_legendre_ex(uint64_t digits, char* out, size_t cap, pimul_mul_fn backend, uint64_t ntt_threshold,
                               uint32_t flags, double* phase_ms, uint64_t* ntt_products);

/* Transform plan for a product: N and the number of HBM passes per transform.
 * Mirrors the sizing of crates/bignum/src/ntt.rs:810-813. */
int pimul_plan(size_t la, size_t lb, uint64_t* n_transform, int* passes);

/* Kernel launch statistics (this engine's own instrumentation; the
 * reference's counterpart is its perf JSONL recorder,
 * crates/pi-core/src/perf.rs).  Launch counts are always kept; with
 * pimul_stats_enable(1) every launch is also timed with CUDA events on its
 * stream.  kclass indexes the kernel classes 0 .. n-1; an out-of-range
 * index returns PIMUL_EINVAL, so callers can enumerate them. */
int pimul_stats_enable(int on);
int pimul_stats_reset(void);
int pimul_stats_get(int kclass, const char** name, uint64_t* launches, uint64_t* timed_launches,
                    double* total_ms);

/*
 * Batched BBP hex digits of pi: digits[i] = the 8 hex digits starting at
 * fractional position positions[i], packed with the first digit in the top
 * nibble (positions[0] == 0 gives 0x243F6A88).  Bit-identical to the
 * reference's extractor; positions must be <= 2^31.  When `stop` is not
 * NULL the call polls *stop and, once it reads non-zero, stops the kernels
 * early and returns PIMUL_ECANCELED (digits untouched).
 *
 * Replaces: crates/pi-core/src/bbp.rs:52 `hex_digits_at(n: u64) -> u32` and
 * bbp.rs:63 `hex_digits_at_interruptible(n, stop: &AtomicBool) -> Option<u32>`,
 * one call per position in crates/pi-cli/src/verify_hex.rs:811-861.
 */
int pimul_bbp_hex_digits(const uint64_t* positions, size_t count, uint32_t* digits,
                         const volatile int* stop);
const char* pimul_bbp_last_error(void);

/* The reference's two modular building blocks on the device, for checking:
 * pow16[i] = 16^e[i] mod d[i] and frac[i] = floor(p[i] 2^64 / d[i]) for
 * 1 <= d[i] < 2^34 and p[i] < d[i] (bbp.rs:117-140).  The series kernel
 * computes their composition as one division-free term (pimul_bbp_terms).
 * Synchronous. */
int pimul_bbp_modops(const uint64_t* e, const uint64_t* d, const uint64_t* p, size_t n, uint64_t* pow16,
                     uint64_t* frac);

/* The term the extractor sums, out[i] = floor((16^e[i] mod d[i]) 2^64 / d[i])
 * (bbp.rs:117-140), computed as the device computes it (an exact 2-adic
 * quotient, no division) for 1 <= d[i] < 2^34, e[i] < 2^40.  For checking;
 * synchronous. */
int pimul_bbp_terms(const uint64_t* e, const uint64_t* d, size_t n, uint64_t* out);

/* Synchronise the calling thread's own stream. */
int pimul_sync(void);

#ifdef __cplusplus
}
#endif

#endif /* PIMUL_H */
