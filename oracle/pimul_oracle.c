/*
 * CPU oracle for the big-integer multiply hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is a plain-C restatement of the
 * reference's CPU algorithm (joelodom/pi, crates/bignum) used as the checker
 * for the CUDA engine and as the timed CPU baseline.  Nothing in the product
 * (pi_gb300/, include/) links or calls it.
 *
 * Each function cites the reference function it restates.  Parallel loops
 * use OpenMP in place of rayon's par_chunks / join; they change scheduling
 * only, never bits.
 */
#include <stdint.h>
#include <stddef.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef unsigned __int128 u128;

/* ------------------------------------------------------------------ */
/* Knobs: crates/bignum/src/config.rs:94-127 (defaults)                */
/* ------------------------------------------------------------------ */
static size_t cfg_karatsuba_threshold = 32;            /* config.rs:101 */
static size_t cfg_parallel_karatsuba_threshold = 512;  /* config.rs:102 */
static size_t cfg_ntt_threshold = 8192;                /* config.rs:103 */
static size_t cfg_four_step_threshold = (size_t)1 << 25; /* config.rs:124 */
static int cfg_threads = 0; /* 0 = OpenMP default */

void orc_set_thresholds(size_t karatsuba, size_t parallel_karatsuba,
                        size_t ntt, size_t four_step) {
  cfg_karatsuba_threshold = karatsuba;
  cfg_parallel_karatsuba_threshold = parallel_karatsuba;
  cfg_ntt_threshold = ntt;
  cfg_four_step_threshold = four_step;
}

void orc_set_threads(int n) {
  cfg_threads = n;
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#endif
}

int orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* ------------------------------------------------------------------ */
/* Goldilocks field: crates/bignum/src/ntt.rs:159-284                  */
/* ------------------------------------------------------------------ */
#define GL_P 0xFFFFFFFF00000001ull   /* ntt.rs:164 */
#define GL_EPS 0xFFFFFFFFull          /* ntt.rs:168 */
#define GL_GEN 7ull                   /* ntt.rs:172 */

static inline uint64_t gl_canon(uint64_t x) { return x >= GL_P ? x - GL_P : x; } /* ntt.rs:177-179 */

/* ntt.rs:183-189: on u64 overflow add EPSILON, then canonicalize. */
uint64_t orc_gl_add(uint64_t a, uint64_t b) {
  uint64_t s = a + b;
  if (s < a) s += GL_EPS;
  return gl_canon(s);
}

/* ntt.rs:193-204: on borrow subtract EPSILON. */
uint64_t orc_gl_sub(uint64_t a, uint64_t b) {
  uint64_t d = a - b;
  if (a < b) d -= GL_EPS;
  return d;
}

/* ntt.rs:218-252: x_lo - x_hi_hi + x_hi_lo * EPSILON, each step fixed up. */
uint64_t orc_gl_reduce128(uint64_t lo, uint64_t hi) {
  uint64_t hh = hi >> 32, hl = hi & 0xFFFFFFFFull;
  uint64_t t0 = lo - hh;
  if (lo < hh) t0 -= GL_EPS;
  t0 = gl_canon(t0);
  uint64_t t1 = hl * GL_EPS;
  uint64_t r = t0 + t1;
  if (r < t0) r += GL_EPS;
  return gl_canon(r);
}

/* ntt.rs:213-216 */
uint64_t orc_gl_mul(uint64_t a, uint64_t b) {
  u128 x = (u128)a * b;
  return orc_gl_reduce128((uint64_t)x, (uint64_t)(x >> 64));
}

/* ntt.rs:255-267 */
uint64_t orc_gl_pow(uint64_t base, uint64_t e) {
  uint64_t acc = 1;
  while (e) {
    if (e & 1) acc = orc_gl_mul(acc, base);
    e >>= 1;
    if (e) base = orc_gl_mul(base, base);
  }
  return acc;
}

/* ntt.rs:272-275 (Fermat) */
uint64_t orc_gl_inv(uint64_t a) { return orc_gl_pow(a, GL_P - 2); }

/* ntt.rs:279-284 */
uint64_t orc_gl_root(uint64_t n) { return orc_gl_pow(GL_GEN, (GL_P - 1) / n); }

/* ------------------------------------------------------------------ */
/* Radix-2 DIT NTT: ntt.rs:286-480                                      */
/* ------------------------------------------------------------------ */
static unsigned log2_exact(size_t n) {
  unsigned k = 0;
  while (((size_t)1 << k) < n) k++;
  return k;
}

static inline uint64_t bitrev(uint64_t i, unsigned bits) {
  uint64_t r = 0;
  for (unsigned b = 0; b < bits; b++) { r = (r << 1) | (i & 1); i >>= 1; }
  return r;
}

/* ntt.rs:300-361 (serial and parallel variants give the same permutation) */
void orc_bit_reverse(uint64_t* a, size_t n) {
  unsigned lg = log2_exact(n);
  if (lg == 0) return;
#pragma omp parallel for schedule(static) if (n >= ((size_t)1 << 18))
  for (size_t i = 0; i < n; i++) {
    size_t j = (size_t)bitrev(i, lg);
    if (i < j) { uint64_t t = a[i]; a[i] = a[j]; a[j] = t; }
  }
}

/* ntt.rs:482-549 plus the per-pass twiddle cache at ntt.rs:569-611:
 * twiddle table of `count` successive powers of omega_len (or its inverse). */
static uint64_t* build_twiddles(size_t count, int inverse) {
  uint64_t* t = (uint64_t*)malloc((count ? count : 1) * sizeof(uint64_t));
  size_t len = count * 2 < 2 ? 2 : count * 2;
  uint64_t w = orc_gl_root(len);
  if (inverse) w = orc_gl_inv(w);
  /* Chunked recurrence: chunk c starts at w^(c*chunk); identical values to
   * the serial chain (ntt.rs:524-549). */
  size_t chunk = 4096;
  size_t nchunks = (count + chunk - 1) / chunk;
  uint64_t wc = orc_gl_pow(w, chunk);
#pragma omp parallel for schedule(static) if (count >= 8192)
  for (size_t c = 0; c < nchunks; c++) {
    uint64_t x = orc_gl_pow(wc, c);
    size_t end = (c + 1) * chunk < count ? (c + 1) * chunk : count;
    for (size_t i = c * chunk; i < end; i++) { t[i] = x; x = orc_gl_mul(x, w); }
  }
  return t;
}

/* Twiddle cache keyed by (count, inverse), tables up to 2^28 entries kept for
 * the life of the process: ntt.rs:569-611. */
static uint64_t* tw_cache[2][64];

static const uint64_t* get_twiddles(size_t count, int inverse, int* owned) {
  unsigned lg = log2_exact(count);
  *owned = 0;
  if (count > ((size_t)1 << 28)) { *owned = 1; return build_twiddles(count, inverse); }
  uint64_t* t;
#pragma omp atomic read
  t = tw_cache[inverse][lg];
  if (t) return t;
  uint64_t* built = build_twiddles(count, inverse);
#pragma omp critical(orc_twiddle_cache)
  {
    if (!tw_cache[inverse][lg]) { tw_cache[inverse][lg] = built; built = 0; }
    t = tw_cache[inverse][lg];
  }
  if (built) free(built);
  return t;
}

/* ntt.rs:406-480: log2(n) passes of CT butterflies with per-pass tables. */
static void butterflies(uint64_t* a, size_t n, int inverse) {
  for (size_t len = 2; len <= n; len *= 2) {
    size_t half = len / 2;
    int owned;
    const uint64_t* tw = get_twiddles(half, inverse, &owned);
    size_t groups = n / len;
    if (groups >= 64 || half < 4096) {
#pragma omp parallel for schedule(static) if (n >= 4096)
      for (size_t g = 0; g < groups; g++) {
        uint64_t* c = a + g * len;
        for (size_t j = 0; j < half; j++) {
          uint64_t u = c[j], t = orc_gl_mul(tw[j], c[j + half]);
          c[j] = orc_gl_add(u, t);
          c[j + half] = orc_gl_sub(u, t);
        }
      }
    } else {
      for (size_t g = 0; g < groups; g++) {
        uint64_t* c = a + g * len;
#pragma omp parallel for schedule(static)
        for (size_t j = 0; j < half; j++) {
          uint64_t u = c[j], t = orc_gl_mul(tw[j], c[j + half]);
          c[j] = orc_gl_add(u, t);
          c[j + half] = orc_gl_sub(u, t);
        }
      }
    }
    if (owned) free((void*)tw);
  }
}

/* ntt.rs:367-373 */
void orc_ntt_forward(uint64_t* a, size_t n) {
  orc_bit_reverse(a, n);
  butterflies(a, n, 0);
}

/* ntt.rs:376-391: inverse butterflies then scale by n^-1. */
void orc_ntt_inverse(uint64_t* a, size_t n) {
  orc_bit_reverse(a, n);
  butterflies(a, n, 1);
  uint64_t ni = orc_gl_inv((uint64_t)n);
#pragma omp parallel for schedule(static) if (n >= 1024)
  for (size_t i = 0; i < n; i++) a[i] = orc_gl_mul(a[i], ni);
}

/* ------------------------------------------------------------------ */
/* Four-step / six-step: ntt.rs:905-1105                                */
/* ------------------------------------------------------------------ */
static void transpose(uint64_t* a, size_t rows, size_t cols) {
  size_t n = rows * cols;
  uint64_t* s = (uint64_t*)malloc(n * sizeof(uint64_t));
#pragma omp parallel for schedule(static) if (n >= 4096)
  for (size_t r = 0; r < rows; r++)
    for (size_t c = 0; c < cols; c++) s[c * rows + r] = a[r * cols + c];
  memcpy(a, s, n * sizeof(uint64_t));
  free(s);
}

/* ntt.rs:1071-1104: position (s, i) of the n2 x n1 matrix times w^(s*i). */
static void cross_twiddle(uint64_t* a, size_t n, size_t n1, size_t n2, int inverse) {
  uint64_t w = orc_gl_root(n);
  if (inverse) w = orc_gl_inv(w);
#pragma omp parallel for schedule(static) if (n >= 4096)
  for (size_t s = 0; s < n2; s++) {
    uint64_t step = orc_gl_pow(w, s), tw = 1;
    uint64_t* row = a + s * n1;
    for (size_t i = 0; i < n1; i++) { row[i] = orc_gl_mul(row[i], tw); tw = orc_gl_mul(tw, step); }
  }
}

static void pick_factorization(size_t n, size_t* n1, size_t* n2) { /* ntt.rs:940-948 */
  unsigned lg = log2_exact(n);
  *n1 = (size_t)1 << (lg / 2);
  *n2 = (size_t)1 << (lg - lg / 2);
}

/* ntt.rs:958-976 */
void orc_four_step_forward(uint64_t* a, size_t n) {
  if (n <= 1) return;
  size_t n1, n2;
  pick_factorization(n, &n1, &n2);
  transpose(a, n1, n2);
#pragma omp parallel for schedule(static)
  for (size_t r = 0; r < n2; r++) orc_ntt_forward(a + r * n1, n1);
  cross_twiddle(a, n, n1, n2, 0);
  transpose(a, n2, n1);
#pragma omp parallel for schedule(static)
  for (size_t r = 0; r < n1; r++) orc_ntt_forward(a + r * n2, n2);
}

/* ntt.rs:982-1000 */
void orc_four_step_inverse(uint64_t* a, size_t n) {
  if (n <= 1) return;
  size_t n1, n2;
  pick_factorization(n, &n1, &n2);
#pragma omp parallel for schedule(static)
  for (size_t r = 0; r < n1; r++) orc_ntt_inverse(a + r * n2, n2);
  transpose(a, n1, n2);
  cross_twiddle(a, n, n1, n2, 1);
#pragma omp parallel for schedule(static)
  for (size_t r = 0; r < n2; r++) orc_ntt_inverse(a + r * n1, n1);
  transpose(a, n2, n1);
}

/* ------------------------------------------------------------------ */
/* Pack / unpack: ntt.rs:626-791                                        */
/* ------------------------------------------------------------------ */
/* ntt.rs:640-665: limb -> four 16-bit coefficients, zero tail. */
void orc_pack(const uint64_t* limbs, size_t nl, uint64_t* coeffs, size_t nc) {
#pragma omp parallel for schedule(static) if (nl >= 1024)
  for (size_t i = 0; i < nl; i++) {
    uint64_t l = limbs[i];
    coeffs[4 * i + 0] = l & 0xFFFF;
    coeffs[4 * i + 1] = (l >> 16) & 0xFFFF;
    coeffs[4 * i + 2] = (l >> 32) & 0xFFFF;
    coeffs[4 * i + 3] = (l >> 48) & 0xFFFF;
  }
  if (nc > 4 * nl) memset(coeffs + 4 * nl, 0, (nc - 4 * nl) * sizeof(uint64_t));
}

/* ntt.rs:686-717 / 723-791 (chunk fold plus serial carry merge).  Writes
 * the trimmed limb vector to out (capacity cap); returns its length, or
 * (size_t)-1 if cap is too small. */
static size_t unpack_chunk(const uint64_t* c, size_t n, uint64_t* out, u128* carry_out) {
  u128 carry = 0;
  size_t k = 0;
  for (size_t i = 0; i < n;) {
    for (unsigned off = 0; off < 4 && i < n; off++, i++) carry += (u128)c[i] << (16 * off);
    out[k++] = (uint64_t)carry;
    carry >>= 64;
  }
  *carry_out = carry;
  return k;
}

size_t orc_unpack(const uint64_t* coeffs, size_t n, uint64_t* out, size_t cap) {
  if (n == 0) return 0;
  size_t nblocks = (n + 3) / 4;
  size_t need = nblocks + 2;
  uint64_t* tmp = (uint64_t*)malloc(need * sizeof(uint64_t));
  size_t len = 0;
  if (n < ((size_t)1 << 20)) { /* ntt.rs:686-717 serial */
    u128 carry;
    len = unpack_chunk(coeffs, n, tmp, &carry);
    while (carry) { tmp[len++] = (uint64_t)carry; carry >>= 64; }
  } else { /* ntt.rs:723-791 parallel chunks + serial merge */
    size_t total_blocks = n / 4;
    int nth = orc_max_threads();
    size_t nchunks = total_blocks < (size_t)nth ? total_blocks : (size_t)nth;
    if (nchunks == 0) nchunks = 1;
    size_t bpc = (total_blocks + nchunks - 1) / nchunks;
    size_t cpc = bpc * 4;
    size_t real_chunks = (n + cpc - 1) / cpc;
    u128* res = (u128*)malloc(real_chunks * sizeof(u128));
    size_t* cnt = (size_t*)malloc(real_chunks * sizeof(size_t));
#pragma omp parallel for schedule(static)
    for (size_t ci = 0; ci < real_chunks; ci++) {
      size_t st = ci * cpc, en = st + cpc < n ? st + cpc : n;
      cnt[ci] = unpack_chunk(coeffs + st, en - st, tmp + ci * bpc, &res[ci]);
    }
    u128 spare = 0;
    for (size_t ci = 0; ci < real_chunks; ci++) {
      for (size_t j = 0; j < cnt[ci]; j++) {
        u128 s = (u128)tmp[ci * bpc + j] + spare;
        tmp[len++] = (uint64_t)s; /* len <= ci*bpc + j: in-place compaction is safe */
        spare = s >> 64;
      }
      spare += res[ci];
    }
    while (spare) { tmp[len++] = (uint64_t)spare; spare >>= 64; }
    free(res); free(cnt);
  }
  while (len && tmp[len - 1] == 0) len--;
  if (len > cap) { free(tmp); return (size_t)-1; }
  memcpy(out, tmp, len * sizeof(uint64_t));
  free(tmp);
  return len;
}

/* ------------------------------------------------------------------ */
/* mul_mag_ntt: ntt.rs:806-865                                          */
/* ------------------------------------------------------------------ */
static size_t next_pow2(size_t x) { size_t p = 1; while (p < x) p <<= 1; return p; }

size_t orc_mul_mag_ntt(const uint64_t* a, size_t la, const uint64_t* b, size_t lb,
                       uint64_t* out, size_t cap) {
  if (la == 0 || lb == 0) return 0;
  size_t n_out = 4 * la + 4 * lb - 1;   /* ntt.rs:810-812 */
  size_t n = next_pow2(n_out);           /* ntt.rs:813 */
  uint64_t* pa = (uint64_t*)malloc(n * sizeof(uint64_t));
  uint64_t* pb = (uint64_t*)malloc(n * sizeof(uint64_t));
  orc_pack(a, la, pa, n);
  orc_pack(b, lb, pb, n);
  int four = n >= cfg_four_step_threshold;  /* ntt.rs:834 */
  if (four) { orc_four_step_forward(pa, n); orc_four_step_forward(pb, n); }
  else { orc_ntt_forward(pa, n); orc_ntt_forward(pb, n); }
#pragma omp parallel for schedule(static) if (n >= 1024)
  for (size_t i = 0; i < n; i++) pa[i] = orc_gl_mul(pa[i], pb[i]);   /* ntt.rs:845-853 */
  free(pb);
  if (four) orc_four_step_inverse(pa, n); else orc_ntt_inverse(pa, n);
  size_t len = orc_unpack(pa, n_out, out, cap);   /* ntt.rs:864 */
  free(pa);
  return len;
}

/* ------------------------------------------------------------------ */
/* Multiply dispatch, schoolbook, Karatsuba: integer.rs:429-643         */
/* ------------------------------------------------------------------ */
static size_t trim(const uint64_t* x, size_t n) { while (n && x[n - 1] == 0) n--; return n; }

/* integer.rs:492-520 */
size_t orc_schoolbook(const uint64_t* a, size_t la, const uint64_t* b, size_t lb,
                      uint64_t* out, size_t cap) {
  if (la == 0 || lb == 0) return 0;
  size_t n = la + lb;
  uint64_t* o = (uint64_t*)calloc(n, sizeof(uint64_t));
  for (size_t i = 0; i < la; i++) {
    u128 carry = 0;
    for (size_t j = 0; j < lb; j++) {
      u128 cur = (u128)o[i + j] + (u128)a[i] * b[j] + carry;
      o[i + j] = (uint64_t)cur;
      carry = cur >> 64;
    }
    size_t k = i + lb;
    while (carry) { u128 cur = (u128)o[k] + carry; o[k] = (uint64_t)cur; carry = cur >> 64; k++; }
  }
  size_t len = trim(o, n);
  if (len > cap) { free(o); return (size_t)-1; }
  memcpy(out, o, len * sizeof(uint64_t));
  free(o);
  return len;
}

/* integer.rs:351-365 (add_mag); result normalized. out needs max(la,lb)+1. */
static size_t add_mag(const uint64_t* a, size_t la, const uint64_t* b, size_t lb, uint64_t* out) {
  if (la < lb) { const uint64_t* t = a; a = b; b = t; size_t tl = la; la = lb; lb = tl; }
  u128 carry = 0;
  for (size_t i = 0; i < la; i++) {
    u128 s = (u128)a[i] + (i < lb ? b[i] : 0) + carry;
    out[i] = (uint64_t)s; carry = s >> 64;
  }
  size_t len = la;
  if (carry) out[len++] = (uint64_t)carry;
  return len;
}

/* integer.rs:368-389 (sub_mag, a >= b) */
static size_t sub_mag(const uint64_t* a, size_t la, const uint64_t* b, size_t lb, uint64_t* out) {
  uint64_t borrow = 0;
  for (size_t i = 0; i < la; i++) {
    uint64_t bi = i < lb ? b[i] : 0;
    uint64_t d = a[i] - bi - borrow;
    borrow = (a[i] < bi) || (a[i] - bi < borrow);
    out[i] = d;
  }
  return trim(out, la);
}

/* integer.rs:612-635 (add_at): dest += src << (64*offset) */
static void add_at(uint64_t* dest, size_t dlen, const uint64_t* src, size_t sl, size_t off) {
  u128 carry = 0;
  size_t i;
  for (i = 0; i < sl; i++) {
    u128 s = (u128)dest[off + i] + src[i] + carry;
    dest[off + i] = (uint64_t)s; carry = s >> 64;
  }
  for (size_t k = off + sl; carry && k < dlen; k++) {
    u128 s = (u128)dest[k] + carry;
    dest[k] = (uint64_t)s; carry = s >> 64;
  }
}

static size_t mul_mag_dispatch(const uint64_t* a, size_t la, const uint64_t* b, size_t lb,
                               uint64_t* out, size_t cap, size_t ntt_max_coeffs);

/* integer.rs:552-608 */
static size_t karatsuba(const uint64_t* a, size_t la, const uint64_t* b, size_t lb,
                        uint64_t* out, size_t cap, size_t ntt_max_coeffs) {
  size_t n = la > lb ? la : lb;
  size_t m = n / 2;
  size_t ma = m < la ? m : la, mb = m < lb ? m : lb;
  const uint64_t *a_lo = a, *a_hi = a + ma, *b_lo = b, *b_hi = b + mb;
  /* Halves are not re-normalised, as in integer.rs:561-562. */
  size_t la_lo = ma, la_hi = la - ma, lb_lo = mb, lb_hi = lb - mb;
  size_t cap0 = la_lo + lb_lo + 1, cap2 = la_hi + lb_hi + 1;
  uint64_t* z0 = (uint64_t*)malloc((cap0 + 1) * 8);
  uint64_t* z2 = (uint64_t*)malloc((cap2 + 1) * 8);
  uint64_t* as = (uint64_t*)malloc((n + 2) * 8);
  uint64_t* bs = (uint64_t*)malloc((n + 2) * 8);
  size_t las = add_mag(a_lo, la_lo, a_hi, la_hi, as);
  size_t lbs = add_mag(b_lo, lb_lo, b_hi, lb_hi, bs);
  size_t cap1 = las + lbs + 1;
  uint64_t* z1 = (uint64_t*)malloc((cap1 + 1) * 8);
  size_t l0, l2, l1;
  int par = (la < lb ? la : lb) >= cfg_parallel_karatsuba_threshold;
#pragma omp parallel sections if (par)
  {
#pragma omp section
    l0 = mul_mag_dispatch(a_lo, la_lo, b_lo, lb_lo, z0, cap0, ntt_max_coeffs);
#pragma omp section
    l2 = mul_mag_dispatch(a_hi, la_hi, b_hi, lb_hi, z2, cap2, ntt_max_coeffs);
#pragma omp section
    l1 = mul_mag_dispatch(as, las, bs, lbs, z1, cap1, ntt_max_coeffs);
  }
  /* z1 = z1_prod - (z0 + z2) */
  size_t ls = (l0 > l2 ? l0 : l2) + 1;
  uint64_t* s02 = (uint64_t*)malloc((ls + 1) * 8);
  size_t l02 = add_mag(z0, l0, z2, l2, s02);
  uint64_t* z1d = (uint64_t*)malloc((l1 + 1) * 8);
  size_t l1d = sub_mag(z1, l1, s02, l02, z1d);
  size_t ol = la + lb + 1;
  uint64_t* o = (uint64_t*)calloc(ol + 1, 8);
  add_at(o, ol, z0, l0, 0);
  add_at(o, ol, z1d, l1d, m);
  add_at(o, ol, z2, l2, 2 * m);
  size_t len = trim(o, ol);
  size_t ret = len;
  if (len > cap) ret = (size_t)-1; else memcpy(out, o, len * 8);
  free(z0); free(z2); free(z1); free(as); free(bs); free(s02); free(z1d); free(o);
  return ret;
}

/* integer.rs:460-486 */
static size_t mul_mag_dispatch(const uint64_t* a, size_t la, const uint64_t* b, size_t lb,
                               uint64_t* out, size_t cap, size_t ntt_max_coeffs) {
  if (la == 0 || lb == 0) return 0;
  size_t smaller = la < lb ? la : lb;
  int fits = (la + lb) * 4 <= ntt_max_coeffs;
  if (fits && smaller >= cfg_ntt_threshold) return orc_mul_mag_ntt(a, la, b, lb, out, cap);
  if (smaller < cfg_karatsuba_threshold) return orc_schoolbook(a, la, b, lb, out, cap);
  return karatsuba(a, la, b, lb, out, cap, ntt_max_coeffs);
}

/* integer.rs:445-453 */
size_t orc_mul_mag(const uint64_t* a, size_t la, const uint64_t* b, size_t lb,
                   uint64_t* out, size_t cap) {
  return mul_mag_dispatch(a, la, b, lb, out, cap, (size_t)1 << 32);
}

/* integer.rs:460 with an explicit NTT size cap (integer.rs:1727-1754). */
size_t orc_mul_mag_dispatch(const uint64_t* a, size_t la, const uint64_t* b, size_t lb,
                            uint64_t* out, size_t cap, size_t ntt_max_coeffs) {
  return mul_mag_dispatch(a, la, b, lb, out, cap, ntt_max_coeffs);
}

/* ------------------------------------------------------------------ */
/* BBP hex digits: crates/pi-core/src/bbp.rs:52-140                     */
/* ------------------------------------------------------------------ */
/* bbp.rs:122-140 */
static uint64_t mod_pow_16(uint64_t e, uint64_t m) {
  if (m == 1) return 0;
  u128 r = 1, base = 16 % m;
  while (e) {
    if (e & 1) r = (r * base) % m;
    e >>= 1;
    if (e) base = (base * base) % m;
  }
  return (uint64_t)r;
}

static void series_tail(uint64_t j, uint64_t n, uint64_t* res);

/* bbp.rs:82-117; stop is polled every 10^4 terms like bbp.rs:88-92.
 * Returns 0 on success, 1 if stopped. */
static int series_fixed(uint64_t j, uint64_t n, const volatile int* stop, uint64_t* res) {
  uint64_t sum = 0;
  for (uint64_t k = 0; k <= n; k++) {
    if (k % 10000 == 0 && stop && *stop) return 1;
    uint64_t d = 8 * k + j;
    uint64_t p = mod_pow_16(n - k, d);
    u128 term = ((u128)p << 64) / d;
    sum += (uint64_t)term;
  }
  uint64_t tail_fixed;
  series_tail(j, n, &tail_fixed);
  *res = sum + tail_fixed;
  return 0;
}

/* bbp.rs:99-115: the f64 tail of the series past k = n, in fixed point. */
static void series_tail(uint64_t j, uint64_t n, uint64_t* res) {
  double tail = 0.0;
  for (int off = 1; off <= 20; off++) {
    uint64_t k = n + (uint64_t)off;
    double denom = (double)(8 * k + j);
    double factor = 1.0;
    for (int q = 0; q < off; q++) factor *= 16.0; /* 16^off is exact in f64 */
    double term = 1.0 / (factor * denom);
    if (term == 0.0) break;
    tail += term;
  }
  *res = (uint64_t)(tail * 18446744073709551616.0);
}

/* bbp.rs:63-80: returns 0 and the packed digits, or 1 when stopped. */
int orc_bbp_hex_digits_at(uint64_t n, const volatile int* stop, uint32_t* digits) {
  uint64_t s1, s4, s5, s6;
  if (series_fixed(1, n, stop, &s1)) return 1;
  if (series_fixed(4, n, stop, &s4)) return 1;
  if (series_fixed(5, n, stop, &s5)) return 1;
  if (series_fixed(6, n, stop, &s6)) return 1;
  uint64_t c = 4 * s1 - 2 * s4 - s5 - s6;
  *digits = (uint32_t)(c >> 32);
  return 0;
}

/* One deep position with each series' terms split across the OpenMP
 * threads: the series sum is wrapping u64 addition (bbp.rs:93-97), which is
 * associative and commutative, so any split gives the same bits as
 * series_fixed.  Only the scheduling differs from bbp.rs:82-117. */
static uint64_t series_fixed_par(uint64_t j, uint64_t n) {
  uint64_t sum = 0;
#pragma omp parallel for schedule(static, 65536) reduction(+ : sum)
  for (int64_t k = 0; k <= (int64_t)n; k++) {
    uint64_t d = 8 * (uint64_t)k + j;
    uint64_t p = mod_pow_16(n - (uint64_t)k, d);
    u128 term = ((u128)p << 64) / d;
    sum += (uint64_t)term;
  }
  uint64_t tail_sum;
  series_tail(j, n, &tail_sum);
  return sum + tail_sum;
}

uint32_t orc_bbp_hex_digits_deep(uint64_t n) {
  uint64_t s1 = series_fixed_par(1, n), s4 = series_fixed_par(4, n);
  uint64_t s5 = series_fixed_par(5, n), s6 = series_fixed_par(6, n);
  uint64_t c = 4 * s1 - 2 * s4 - s5 - s6;
  return (uint32_t)(c >> 32);
}

/* Many positions across threads (the verify-hex check loop's shape). */
void orc_bbp_batch(const uint64_t* pos, size_t n, uint32_t* out) {
#pragma omp parallel for schedule(dynamic, 1)
  for (size_t i = 0; i < n; i++) orc_bbp_hex_digits_at(pos[i], 0, &out[i]);
}

/* Adapter with the engine's C-ABI multiply signature (include/pimul.h
 * pimul_mul_fn): lets a host driver use this CPU restatement as its
 * multiply backend (the reference's own CPU multiply path). */
int orc_mul_abi(const uint64_t* a, size_t la, const uint64_t* b, size_t lb,
                uint64_t* out, size_t cap, size_t* out_len) {
  size_t n = orc_mul_mag_ntt(a, la, b, lb, out, cap);
  if (n == (size_t)-1) return 1;
  *out_len = n;
  return 0;
}
