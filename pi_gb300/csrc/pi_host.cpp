// Host side above the C ABI: the reference's pi pipeline restated in C++,
// with every large product routed through the GPU multiply.
//
// This is the caller of the drop-in (crates/bignum/src/integer.rs:445
// mul_mag -> ntt.rs:806 mul_mag_ntt) in the three places pi-core uses it:
// Chudnovsky binary splitting, the final assembly's Newton reciprocal and
// square root, and the decimal conversion's Newton divisions.  It mirrors
// the reference's algorithms and thresholds:
//   * mul_mag dispatch: schoolbook below 32 limbs, Karatsuba below the NTT
//     threshold (8192 limbs of the smaller operand), else the NTT multiply
//     (crates/bignum/src/integer.rs:445-608, config.rs:94-127);
//   * Float: sign * mantissa * 2^exp, round-half-up to prec bits
//     (crates/bignum/src/float.rs:524-569), precision-doubling Newton for
//     the reciprocal (float.rs:417-474) and the square root (float.rs:85-174);
//   * Integer division: Knuth D below 64 limbs, Newton reciprocal above
//     (integer.rs:702-827, 1031-1083); decimal conversion by divide and
//     conquer on powers of ten (integer.rs:892-983);
//   * Chudnovsky: n_terms = ceil(D / 14.1816...) + 8, binary splitting without
//     the root P, pi = 426880 sqrt(10005) Q / (A Q + T), digits by scaling
//     with 10^(D-1) and truncating (crates/pi-core/src/algorithm/
//     chudnovsky.rs:75-413, util.rs:25-83, precision.rs:45-70).
// The multiply backend is pluggable (C ABI pimul_pi_chudnovsky): the GPU
// engine by default, or any function with pimul_mul's signature.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <exception>
#include <functional>
#include <list>
#include <map>
#include <condition_variable>
#include <mutex>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/pimul.h"
#include "dec.h"
#include "leaves.h"
#include "splitmerge.h"
#include "agm.h"

namespace pihost {

typedef unsigned __int128 u128;

// Limb arrays: large blocks (>= 1 MiB) come from a cache of freed blocks,
// so the multi-GB temporaries of the Newton iterations reuse memory that is
// already mapped instead of taking a page fault per 4 KiB each time, and
// resize() without a value does not zero-fill (every such use writes all
// words before reading them).
struct BlockCache {
  std::mutex mu;
  std::multimap<size_t, void*> blocks;  // size class in bytes -> block
  size_t cached = 0;
};
static BlockCache& block_cache() {
  static BlockCache* c = new BlockCache;  // never destroyed: usable during static destruction
  return *c;
}
static const size_t BIG_BYTES = (size_t)1 << 20;
static const size_t CACHE_MAX = (size_t)24 << 30;
static size_t size_class(size_t bytes) {  // round up to an eighth of the next power of two
  size_t p = 1;
  while (p < bytes) p <<= 1;
  size_t step = std::max<size_t>(p >> 3, 64);
  return (bytes + step - 1) / step * step;
}
static void* big_alloc(size_t bytes) {
  const size_t c = size_class(bytes);
  BlockCache& bc = block_cache();
  {
    std::lock_guard<std::mutex> lk(bc.mu);
    auto it = bc.blocks.find(c);
    if (it != bc.blocks.end()) {
      void* p = it->second;
      bc.blocks.erase(it);
      bc.cached -= c;
      return p;
    }
  }
  void* p = std::malloc(c);
  if (!p) throw std::bad_alloc();
  return p;
}
static void big_free(void* p, size_t bytes) {
  const size_t c = size_class(bytes);
  BlockCache& bc = block_cache();
  {
    std::lock_guard<std::mutex> lk(bc.mu);
    if (bc.cached + c <= CACHE_MAX) {
      bc.blocks.emplace(c, p);
      bc.cached += c;
      return;
    }
  }
  std::free(p);
}
template <class T>
struct LimbAlloc {
  using value_type = T;
  LimbAlloc() noexcept {}
  template <class U>
  LimbAlloc(const LimbAlloc<U>&) noexcept {}
  T* allocate(size_t n) {
    const size_t b = n * sizeof(T);
    if (b >= BIG_BYTES) return static_cast<T*>(big_alloc(b));
    T* p = static_cast<T*>(std::malloc(b ? b : 1));
    if (!p) throw std::bad_alloc();
    return p;
  }
  void deallocate(T* p, size_t n) {
    const size_t b = n * sizeof(T);
    if (b >= BIG_BYTES) big_free(p, b);
    else std::free(p);
  }
  template <class U>
  void construct(U* p) noexcept {
    ::new ((void*)p) U;
  }
  template <class U, class... A>
  void construct(U* p, A&&... a) {
    ::new ((void*)p) U(std::forward<A>(a)...);
  }
  template <class U>
  bool operator==(const LimbAlloc<U>&) const noexcept { return true; }
  template <class U>
  bool operator!=(const LimbAlloc<U>&) const noexcept { return false; }
};
using Limbs = std::vector<uint64_t, LimbAlloc<uint64_t>>;

// Host loops over large limb arrays run on all cores.
static const size_t PAR_LIMBS = (size_t)1 << 18;
static void parallel_for(size_t n, const std::function<void(size_t, size_t)>& fn);
static void par_range(size_t n, const std::function<void(size_t, size_t)>& fn) {
  if (n < PAR_LIMBS) {
    fn(0, n);
    return;
  }
  const size_t chunk = (size_t)1 << 16;
  const size_t nchunks = (n + chunk - 1) / chunk;
  parallel_for(nchunks, [&](size_t lo, size_t hi) { fn(lo * chunk, std::min(n, hi * chunk)); });
}
static Limbs copy_limbs(const uint64_t* src, size_t n) {
  Limbs out(n);
  par_range(n, [&](size_t lo, size_t hi) { memcpy(out.data() + lo, src + lo, (hi - lo) * 8); });
  return out;
}

// ------------------------------------------------------------------ config
static size_t g_karatsuba_threshold = 32;   // config.rs:101
static size_t g_newton_div_threshold = 64;  // config.rs:104
static size_t g_to_string_dc_threshold = 32;  // config.rs:105
static const uint64_t PARALLEL_SPLIT = 64;  // pi-core config.rs:61

typedef int (*mul_fn)(const uint64_t*, size_t, const uint64_t*, size_t, uint64_t*, size_t, size_t*);

// ------------------------------------------------------------------ per-call state
// Every driver call (pimul_pi_*, pimul_to_decimal) runs with a context of its
// own: the multiply backend, the NTT threshold, the first backend error and
// the call's statistics.  The calling thread holds it in t_ctx and every
// helper thread the pipeline starts (Worker, parallel_for) inherits it, so
// calls from different host threads share no mutable state.
struct PiCtx {
  mul_fn backend = nullptr;
  size_t ntt_threshold = 8192;  // config.rs:103
  std::atomic<int> error{0};
  std::atomic<uint64_t> ntt_calls{0};
  std::atomic<uint64_t> ntt_hist[33];
  std::atomic<uint64_t> batch_levels{0};
  double bt[5] = {0, 0, 0, 0, 0};  // level-batched splitting: time per step (PIMUL_PI_TIMING)
  std::mutex bt_mu;                  // segments of the splitting run on two host threads
  double leaf_ms = 0;
  uint64_t serve_nodes = 0;  // > 0: the splitting tree above this many nodes goes through the multiply service
  uint64_t served_requests = 0;
  PiCtx() {
    for (auto& h : ntt_hist) h.store(0);
  }
};
static thread_local PiCtx* t_ctx = nullptr;
static PiCtx& C() {
  static thread_local PiCtx idle;  // only reached outside a driver call
  return t_ctx ? *t_ctx : idle;
}

static void bt_add(int i, double ms) {
  PiCtx& c = C();
  std::lock_guard<std::mutex> lk(c.bt_mu);
  c.bt[i] += ms;
}

// A backend error stops the pipeline at once: mul_ntt throws PiAbort, which
// unwinds to the driver's entry point (threads hand it on at join).
struct PiAbort {
  int rc;
};

// A helper thread that runs with the caller's context and hands an
// exception thrown inside it to whoever joins it.  The destructor joins too,
// so a thread is never left running when its parent unwinds.
class Worker {
 public:
  Worker() = default;
  template <class F>
  explicit Worker(F&& f) {
    start(std::forward<F>(f));
  }
  template <class F>
  void start(F&& f) {
    PiCtx* c = t_ctx;
    th_ = std::thread([this, c, fn = std::forward<F>(f)]() mutable {
      t_ctx = c;
      try {
        fn();
      } catch (...) {
        ex_ = std::current_exception();
      }
    });
  }
  void join() {
    if (th_.joinable()) th_.join();
    if (ex_) {
      std::exception_ptr e = ex_;
      ex_ = nullptr;
      std::rethrow_exception(e);
    }
  }
  ~Worker() {
    if (th_.joinable()) th_.join();
  }
  Worker(const Worker&) = delete;
  Worker& operator=(const Worker&) = delete;

 private:
  std::exception_ptr ex_;
  std::thread th_;
};

// Runs a driver body with ctx as the calling thread's context: returns the
// body's code, the first backend error, or PIMUL_ENOMEM for a failed host
// allocation.
template <class F>
static int with_ctx(PiCtx& ctx, F&& body) {
  PiCtx* prev = t_ctx;
  t_ctx = &ctx;
  int rc;
  try {
    rc = body();
    if (!rc && ctx.error.load()) rc = ctx.error.load();
  } catch (const PiAbort& e) {
    rc = e.rc;
  } catch (const std::bad_alloc&) {
    rc = PIMUL_ENOMEM;
  }
  t_ctx = prev;
  return rc;
}

// ------------------------------------------------------------------ magnitudes
static void trim(Limbs& a) {
  while (!a.empty() && a.back() == 0) a.pop_back();
}

static uint64_t bits_of(const Limbs& a) {
  if (a.empty()) return 0;
  return (a.size() - 1) * 64 + (64 - __builtin_clzll(a.back()));
}

static int cmp_mag(const Limbs& a, const Limbs& b) {
  if (a.size() != b.size()) return a.size() < b.size() ? -1 : 1;
  for (size_t i = a.size(); i-- > 0;)
    if (a[i] != b[i]) return a[i] < b[i] ? -1 : 1;
  return 0;
}

static Limbs add_mag(const Limbs& a, const Limbs& b) {  // integer.rs:351-365
  const Limbs& L = a.size() >= b.size() ? a : b;
  const Limbs& S = a.size() >= b.size() ? b : a;
  Limbs out(L.size() + 1);
  if (L.size() < PAR_LIMBS) {
    u128 c = 0;
    for (size_t i = 0; i < L.size(); i++) {
      c += (u128)L[i] + (i < S.size() ? S[i] : 0);
      out[i] = (uint64_t)c;
      c >>= 64;
    }
    out[L.size()] = (uint64_t)c;
  } else {
    // chunks add with carry-in 0 and record their carry out; the carries
    // are then rippled into the following chunks (rarely past one limb)
    const size_t chunk = (size_t)1 << 16, nch = (L.size() + chunk - 1) / chunk;
    std::vector<uint8_t> cout(nch);
    parallel_for(nch, [&](size_t clo, size_t chi) {
      for (size_t c = clo; c < chi; c++) {
        u128 cy = 0;
        for (size_t i = c * chunk; i < std::min(L.size(), (c + 1) * chunk); i++) {
          cy += (u128)L[i] + (i < S.size() ? S[i] : 0);
          out[i] = (uint64_t)cy;
          cy >>= 64;
        }
        cout[c] = (uint8_t)cy;
      }
    });
    uint64_t carry = 0;
    for (size_t c = 0; c < nch; c++) {
      size_t i = c * chunk, end = std::min(L.size(), (c + 1) * chunk);
      uint64_t cin = carry;
      while (cin && i < end) {
        out[i] += 1;
        cin = out[i] == 0;
        i++;
      }
      carry = cout[c] + cin;
    }
    out[L.size()] = carry;
  }
  trim(out);
  return out;
}

static Limbs sub_mag(const Limbs& a, const Limbs& b) {  // a >= b, integer.rs:368-389
  Limbs out(a.size());
  if (a.size() < PAR_LIMBS) {
    uint64_t borrow = 0;
    for (size_t i = 0; i < a.size(); i++) {
      uint64_t bi = i < b.size() ? b[i] : 0;
      uint64_t d = a[i] - bi - borrow;
      borrow = (a[i] < bi) || (a[i] - bi < borrow);
      out[i] = d;
    }
  } else {
    const size_t chunk = (size_t)1 << 16, nch = (a.size() + chunk - 1) / chunk;
    std::vector<uint8_t> bout(nch);
    parallel_for(nch, [&](size_t clo, size_t chi) {
      for (size_t c = clo; c < chi; c++) {
        uint64_t borrow = 0;
        for (size_t i = c * chunk; i < std::min(a.size(), (c + 1) * chunk); i++) {
          uint64_t bi = i < b.size() ? b[i] : 0;
          uint64_t d = a[i] - bi - borrow;
          borrow = (a[i] < bi) || (a[i] - bi < borrow);
          out[i] = d;
        }
        bout[c] = (uint8_t)borrow;
      }
    });
    uint64_t borrow = 0;
    for (size_t c = 0; c < nch; c++) {
      size_t i = c * chunk, end = std::min(a.size(), (c + 1) * chunk);
      uint64_t bin = borrow;
      while (bin && i < end) {
        bin = out[i] == 0;
        out[i] -= 1;
        i++;
      }
      borrow = bout[c] + bin;
    }
  }
  trim(out);
  return out;
}

static Limbs shl_mag(const Limbs& a, uint64_t s) {  // integer.rs:1097-1125
  if (a.empty()) return {};
  const size_t w = s / 64, r = s % 64, n = a.size() + w + 1;
  Limbs out(n);
  par_range(n, [&](size_t lo, size_t hi) {
    for (size_t k = lo; k < hi; k++) {
      // out[k] = a[k - w] << r | a[k - w - 1] >> (64 - r)
      uint64_t v = 0;
      if (k >= w && k - w < a.size()) v = a[k - w] << r;
      if (r && k >= w + 1 && k - w - 1 < a.size()) v |= a[k - w - 1] >> (64 - r);
      out[k] = v;
    }
  });
  trim(out);
  return out;
}

static Limbs shr_mag(const Limbs& a, uint64_t s) {  // integer.rs:1127-1155
  size_t w = s / 64, r = s % 64;
  if (w >= a.size()) return {};
  Limbs out(a.size() - w);
  par_range(out.size(), [&](size_t lo, size_t hi) {
    for (size_t i = lo; i < hi; i++) {
      uint64_t v = a[i + w] >> r;
      uint64_t h = (r && i + w + 1 < a.size()) ? a[i + w + 1] << (64 - r) : 0;
      out[i] = v | h;
    }
  });
  trim(out);
  return out;
}

static bool has_low_bits(const Limbs& a, uint64_t n) {  // float.rs:615-634
  if (n == 0 || a.empty()) return false;
  size_t full = n / 64;
  for (size_t i = 0; i < full && i < a.size(); i++)
    if (a[i]) return true;
  unsigned r = n % 64;
  if (r && full < a.size() && (a[full] & ((1ull << r) - 1))) return true;
  return false;
}

static uint64_t bit_at(const Limbs& a, uint64_t i) {
  size_t l = i / 64;
  return l < a.size() ? (a[l] >> (i % 64)) & 1 : 0;
}

// ------------------------------------------------------------------ multiply
static Limbs mul_schoolbook(const Limbs& a, const Limbs& b) {  // integer.rs:492-520
  if (a.empty() || b.empty()) return {};
  Limbs out(a.size() + b.size(), 0);
  for (size_t i = 0; i < a.size(); i++) {
    u128 carry = 0;
    for (size_t j = 0; j < b.size(); j++) {
      u128 cur = (u128)out[i + j] + (u128)a[i] * b[j] + carry;
      out[i + j] = (uint64_t)cur;
      carry = cur >> 64;
    }
    size_t k = i + b.size();
    while (carry) {
      u128 cur = (u128)out[k] + carry;
      out[k] = (uint64_t)cur;
      carry = cur >> 64;
      k++;
    }
  }
  trim(out);
  return out;
}

static Limbs mul_mag(const Limbs& a, const Limbs& b);

static void add_at(Limbs& d, const Limbs& s, size_t off) {  // integer.rs:612-635
  if (s.empty()) return;
  if (d.size() < off + s.size()) d.resize(off + s.size(), 0);
  u128 c = 0;
  for (size_t i = 0; i < s.size(); i++) {
    c += (u128)d[off + i] + s[i];
    d[off + i] = (uint64_t)c;
    c >>= 64;
  }
  for (size_t k = off + s.size(); c; k++) {
    if (k >= d.size()) d.push_back(0);
    c += d[k];
    d[k] = (uint64_t)c;
    c >>= 64;
  }
}

static Limbs mul_karatsuba(const Limbs& a, const Limbs& b) {  // integer.rs:552-608
  size_t n = std::max(a.size(), b.size()), m = n / 2;
  Limbs alo(a.begin(), a.begin() + std::min(m, a.size())), ahi(a.begin() + std::min(m, a.size()), a.end());
  Limbs blo(b.begin(), b.begin() + std::min(m, b.size())), bhi(b.begin() + std::min(m, b.size()), b.end());
  Limbs z0 = mul_mag(alo, blo);
  Limbs z2 = mul_mag(ahi, bhi);
  Limbs as = alo, bs = blo;
  trim(as);
  trim(bs);
  Limbs ah = ahi, bh = bhi;
  trim(ah);
  trim(bh);
  Limbs z1 = mul_mag(add_mag(as, ah), add_mag(bs, bh));
  Limbs z02 = add_mag(z0, z2);
  z1 = sub_mag(z1, z02);
  Limbs out(a.size() + b.size() + 1, 0);
  add_at(out, z0, 0);
  add_at(out, z1, m);
  add_at(out, z2, 2 * m);
  trim(out);
  return out;
}

static Limbs mul_ntt(const Limbs& a, const Limbs& b) {
  Limbs out(a.size() + b.size());
  size_t n = 0;
  PiCtx& c = C();
  if (int e = c.error.load()) throw PiAbort{e};
  int rc = c.backend ? c.backend(a.data(), a.size(), b.data(), b.size(), out.data(), out.size(), &n)
                     : pimul_mul(a.data(), a.size(), b.data(), b.size(), out.data(), out.size(), &n);
  if (rc) {
    int none = 0;
    c.error.compare_exchange_strong(none, rc);
    throw PiAbort{rc};
  }
  uint64_t L = 0;
  while ((1ull << L) < 4 * (a.size() + b.size()) - 1) L++;
  C().ntt_calls.fetch_add(1, std::memory_order_relaxed);
  C().ntt_hist[L].fetch_add(1, std::memory_order_relaxed);
  out.resize(n);
  return out;
}

// integer.rs:460-486 (with the 2^32-coefficient cap of integer.rs:445-453)
static Limbs mul_mag(const Limbs& a0, const Limbs& b0) {
  if (a0.empty() || b0.empty()) return {};
  size_t smaller = std::min(a0.size(), b0.size());
  bool fits = (a0.size() + b0.size()) * 4 <= (1ull << 32);
  if (fits && smaller >= C().ntt_threshold) return mul_ntt(a0, b0);
  if (smaller < g_karatsuba_threshold) return mul_schoolbook(a0, b0);
  return mul_karatsuba(a0, b0);
}

static Limbs mul_small(const Limbs& a, uint64_t s) {
  if (a.empty() || s == 0) return {};
  Limbs out(a.size() + 1);
  u128 c = 0;
  for (size_t i = 0; i < a.size(); i++) {
    c += (u128)a[i] * s;
    out[i] = (uint64_t)c;
    c >>= 64;
  }
  out[a.size()] = (uint64_t)c;
  trim(out);
  return out;
}

// ------------------------------------------------------------------ Integer
struct Int {
  Limbs m;
  bool neg = false;
  Int() {}
  explicit Int(uint64_t v) {
    if (v) m.push_back(v);
  }
  Int(Limbs l, bool n) : m(std::move(l)), neg(n) {
    trim(m);
    if (m.empty()) neg = false;
  }
  bool zero() const { return m.empty(); }
};

static Int add(const Int& a, const Int& b) {  // integer.rs:391-421
  if (a.neg == b.neg) return Int(add_mag(a.m, b.m), a.neg);
  int c = cmp_mag(a.m, b.m);
  if (c == 0) return Int();
  if (c > 0) return Int(sub_mag(a.m, b.m), a.neg);
  return Int(sub_mag(b.m, a.m), b.neg);
}
static Int neg(Int a) {
  if (!a.zero()) a.neg = !a.neg;
  return a;
}
static Int sub(const Int& a, const Int& b) { return add(a, neg(b)); }
static Int mul(const Int& a, const Int& b) {  // integer.rs:637-643
  return Int(mul_mag(a.m, b.m), a.neg != b.neg);
}
static Int mulu(const Int& a, uint64_t s) { return Int(mul_small(a.m, s), a.neg); }

// Knuth algorithm D (integer.rs:702-827), magnitudes, b nonzero.
static void divrem_knuth(const Limbs& a, const Limbs& b, Limbs& q, Limbs& r) {
  if (cmp_mag(a, b) < 0) {
    q.clear();
    r = a;
    return;
  }
  if (b.size() == 1) {
    q.assign(a.size(), 0);
    u128 rem = 0;
    for (size_t i = a.size(); i-- > 0;) {
      u128 cur = (rem << 64) | a[i];
      q[i] = (uint64_t)(cur / b[0]);
      rem = cur % b[0];
    }
    trim(q);
    r.clear();
    if (rem) r.push_back((uint64_t)rem);
    return;
  }
  size_t n = b.size(), m = a.size() - n;
  int d = __builtin_clzll(b[n - 1]);
  Limbs v = d ? shl_mag(b, d) : b;
  Limbs u = d ? shl_mag(a, d) : a;
  u.resize(a.size() + 1, 0);
  uint64_t vt = v[n - 1], vn = v[n - 2];
  q.assign(m + 1, 0);
  for (size_t j = m + 1; j-- > 0;) {
    u128 num = ((u128)u[j + n] << 64) | u[j + n - 1];
    u128 qhat, rhat;
    if (u[j + n] >= vt) {
      qhat = UINT64_MAX;
      rhat = num - qhat * vt;
    } else {
      qhat = num / vt;
      rhat = num % vt;
    }
    while (rhat < ((u128)1 << 64)) {
      if ((u128)(uint64_t)qhat * vn <= ((rhat << 64) | u[j + n - 2])) break;
      qhat--;
      rhat += vt;
    }
    // u[j..j+n] -= qhat * v
    u128 carry = 0;
    int64_t borrow = 0;
    for (size_t i = 0; i < n; i++) {
      u128 p = (u128)(uint64_t)qhat * v[i] + carry;
      carry = p >> 64;
      __int128 t = (__int128)u[i + j] - (uint64_t)p - borrow;
      borrow = t < 0;
      u[i + j] = (uint64_t)t;
    }
    __int128 t = (__int128)u[j + n] - (__int128)carry - borrow;
    u[j + n] = (uint64_t)t;
    if (t < 0) {  // add back
      qhat--;
      u128 c = 0;
      for (size_t i = 0; i < n; i++) {
        c += (u128)u[i + j] + v[i];
        u[i + j] = (uint64_t)c;
        c >>= 64;
      }
      u[j + n] += (uint64_t)c;
    }
    q[j] = (uint64_t)qhat;
  }
  u.resize(n);
  r = d ? shr_mag(u, d) : u;
  trim(r);
  trim(q);
}

// ------------------------------------------------------------------ Float
struct Flt {
  uint64_t prec = 64;
  bool sign = false;
  Limbs mant;
  int64_t exp = 0;
  bool zero() const { return mant.empty(); }
};

static void round_to_prec(Flt& f) {  // float.rs:524-569 (round half up)
  if (f.mant.empty()) {
    f.sign = false;
    f.exp = 0;
    return;
  }
  uint64_t b = bits_of(f.mant);
  if (b <= f.prec) return;
  uint64_t drop = b - f.prec;
  uint64_t rb = bit_at(f.mant, drop - 1);
  Limbs nl = shr_mag(f.mant, drop);
  if (rb) {  // + 1, in place
    size_t i = 0;
    while (i < nl.size() && ++nl[i] == 0) i++;
    if (i == nl.size()) nl.push_back(1);
  }
  f.mant = std::move(nl);
  f.exp += (int64_t)drop;
  uint64_t nb = bits_of(f.mant);
  if (nb > f.prec) {
    uint64_t extra = nb - f.prec;
    f.mant = shr_mag(f.mant, extra);
    f.exp += (int64_t)extra;
  }
}

static Flt flt_from_u64(uint64_t v, uint64_t prec) {
  Flt f;
  f.prec = prec;
  if (v) f.mant.push_back(v);
  round_to_prec(f);
  return f;
}

static Flt flt_from_int(const Int& v) {  // float.rs From<Integer>
  Flt f;
  f.sign = v.neg;
  f.mant = copy_limbs(v.m.data(), v.m.size());
  f.prec = std::max<uint64_t>(bits_of(v.m), 64);
  return f;
}

static Flt flt_from_f64(double v, uint64_t prec) {  // float.rs:571-593
  Flt f;
  f.prec = prec;
  if (v == 0.0) return f;
  uint64_t bits;
  memcpy(&bits, &v, 8);
  f.sign = (bits >> 63) & 1;
  int64_t raw_exp = (bits >> 52) & 0x7FF;
  uint64_t raw = bits & ((1ull << 52) - 1);
  uint64_t mu;
  if (raw_exp == 0) {
    mu = raw;
    f.exp = -1074;
  } else {
    mu = raw | (1ull << 52);
    f.exp = raw_exp - 1023 - 52;
  }
  f.mant = Limbs{mu};
  trim(f.mant);
  round_to_prec(f);
  return f;
}

static void to_f64_with_exp(const Limbs& a, double& m, int64_t& e) {  // integer.rs:187-215
  uint64_t tb = bits_of(a);
  if (tb <= 53) {
    uint64_t v = a.empty() ? 0 : a[0];
    int64_t x = (int64_t)tb - 1;
    m = (double)v * std::ldexp(1.0, -(int)x);
    e = x;
  } else {
    uint64_t drop = tb - 53;
    Limbs t = shr_mag(a, drop);
    uint64_t top = t.empty() ? 0 : t[0];
    m = (double)top * std::ldexp(1.0, -52);
    e = (int64_t)drop + 52;
  }
}

static Flt truncated_to_prec(const Flt& s, uint64_t prec) {  // float.rs:485-518
  Flt out;
  out.prec = prec;
  if (s.zero()) return out;
  if (bits_of(s.mant) <= prec) {
    out = s;
    out.prec = prec;
    return out;
  }
  size_t keep = (prec + 64) / 64 + 1;
  if (keep >= s.mant.size()) {
    out = s;
    out.prec = prec;
    round_to_prec(out);
    return out;
  }
  size_t drop = s.mant.size() - keep;
  out.sign = s.sign;
  out.mant.assign(s.mant.begin() + drop, s.mant.end());
  out.exp = s.exp + (int64_t)drop * 64;
  round_to_prec(out);
  return out;
}

static Flt mul_at_prec(const Flt& a, const Flt& b, uint64_t prec) {  // float.rs:331-344
  Flt out;
  out.prec = prec;
  if (a.zero() || b.zero()) return out;
  out.mant = mul_mag(a.mant, b.mant);
  out.exp = a.exp + b.exp;
  out.sign = a.sign != b.sign;
  round_to_prec(out);
  return out;
}

static Flt add_at_prec(const Flt& a, const Flt& b, uint64_t prec) {  // float.rs:284-323
  if (a.zero()) {
    Flt r = b;
    r.prec = prec;
    round_to_prec(r);
    return r;
  }
  if (b.zero()) {
    Flt r = a;
    r.prec = prec;
    round_to_prec(r);
    return r;
  }
  // align to the smaller exponent, then a signed add of the magnitudes
  // (integer.rs:391-421) without copying the unshifted operand
  int64_t ae = a.exp, be = b.exp;
  Limbs sa, sb;
  const Limbs* pa = &a.mant;
  const Limbs* pb = &b.mant;
  if (ae > be) {
    sa = shl_mag(a.mant, (uint64_t)(ae - be));
    pa = &sa;
  } else if (be > ae) {
    sb = shl_mag(b.mant, (uint64_t)(be - ae));
    pb = &sb;
  }
  ae = std::min(ae, be);
  Limbs m;
  bool neg = false;
  if (a.sign == b.sign) {
    m = add_mag(*pa, *pb);
    neg = a.sign;
  } else {
    int c = cmp_mag(*pa, *pb);
    if (c > 0) {
      m = sub_mag(*pa, *pb);
      neg = a.sign;
    } else if (c < 0) {
      m = sub_mag(*pb, *pa);
      neg = b.sign;
    }
  }
  Flt out;
  out.prec = prec;
  out.sign = m.empty() ? false : neg;
  out.mant = std::move(m);
  out.exp = ae;
  round_to_prec(out);
  return out;
}

static Flt sub_at_prec(const Flt& a, const Flt& b, uint64_t prec) {
  Flt nb = b;
  if (!nb.zero()) nb.sign = !nb.sign;
  return add_at_prec(a, nb, prec);
}

// Newton reciprocal with precision doubling and one extra iteration at
// the cap (float.rs:417-474).
static Flt reciprocal_at_prec(const Flt& self, uint64_t target) {
  Flt mag = self;
  mag.sign = false;
  double m;
  int64_t e;
  to_f64_with_exp(mag.mant, m, e);
  Flt x = flt_from_f64(1.0 / m, 64);
  x.exp += -(e + mag.exp);
  round_to_prec(x);
  uint64_t cur = 64;
  int full = 0;
  while (true) {
    cur = std::min(cur * 2, target + 16);
    Flt b = truncated_to_prec(mag, cur);
    x.prec = cur;
    round_to_prec(x);
    Flt bx = mul_at_prec(b, x, cur + 8);
    Flt two = flt_from_f64(2.0, cur + 8);
    Flt t = sub_at_prec(two, bx, cur + 8);
    x = mul_at_prec(x, t, cur);
    if (cur >= target + 16 && ++full >= 2) break;
  }
  x.prec = target;
  round_to_prec(x);
  x.sign = self.sign;
  return x;
}

static Flt div_at_prec(const Flt& a, const Flt& b, uint64_t prec) {  // float.rs:360-373
  if (a.zero()) {
    Flt z;
    z.prec = prec;
    return z;
  }
  Flt r = reciprocal_at_prec(b, prec + 16);
  return mul_at_prec(a, r, prec);
}

// Newton square root with precision doubling (float.rs:85-174).
static void sqrt_mut(Flt& self) {
  if (self.zero()) return;
  uint64_t target = self.prec;
  double m;
  int64_t e;
  to_f64_with_exp(self.mant, m, e);
  int64_t tot = e + self.exp;
  int64_t half = tot >= 0 ? tot / 2 : -((-tot + 1) / 2);
  int64_t left = tot - 2 * half;
  double mc = left == 0 ? m : m * 2.0;
  uint64_t cur = 64;
  Flt x = flt_from_f64(std::sqrt(mc), cur);
  x.exp += half;
  round_to_prec(x);
  int full = 0;
  while (true) {
    cur = std::min(cur * 2, target + 16);
    Flt n = truncated_to_prec(self, cur);
    x.prec = cur;
    round_to_prec(x);
    Flt d = div_at_prec(n, x, cur + 8);
    Flt s = add_at_prec(x, d, cur + 8);
    s.exp -= 1;
    s.prec = cur;
    round_to_prec(s);
    x = s;
    if (cur >= target + 16 && ++full >= 2) break;
  }
  x.prec = target;
  round_to_prec(x);
  self = x;
}

// sqrt(n) for a small integer n at prec bits by the multiplication-only
// Newton iteration for 1/sqrt(n), y <- y + y (1 - n y^2) / 2, at doubling
// precision, then sqrt(n) = n y.  Used by the batched form only (the plain
// form keeps the division-based iteration of float.rs:85-174, restated in
// sqrt_mut); the two results agree to within an ulp of the working
// precision, which sits 256 bits below the last digit.
static Flt sqrt_int_fast(uint64_t n, uint64_t prec) {
  const uint64_t target = prec + 64;
  Flt y = flt_from_f64(1.0 / std::sqrt((double)n), 64);
  const Flt nf = flt_from_u64(n, 64);
  const Flt one = flt_from_u64(1, 64);
  uint64_t cur = 48;  // bits right in the f64 start
  while (cur < target) {
    cur = std::min(2 * cur, target);
    const uint64_t w = cur + 32;
    Flt y2 = mul_at_prec(y, y, w);
    Flt e = sub_at_prec(one, mul_at_prec(y2, nf, w), w);  // |e| ~ 2^-(cur/2)
    e = truncated_to_prec(e, cur / 2 + 64);
    Flt c = mul_at_prec(y, e, w);
    c.exp -= 1;
    y = add_at_prec(y, c, w);
  }
  return mul_at_prec(y, nf, prec);
}

// In-place square root of a positive Float by the same multiplication-only
// iteration as sqrt_int_fast (a Newton iteration for 1/sqrt(x) from an f64
// start, then sqrt(x) = x y), for drivers that opt out of the reference's
// division-based sqrt_mut; results agree to within an ulp.
static void sqrt_fast(Flt& self) {
  if (self.zero()) return;
  const uint64_t prec = self.prec, target = prec + 64;
  double m;
  int64_t e;
  to_f64_with_exp(self.mant, m, e);
  const int64_t tot = e + self.exp;  // value = m 2^tot, m in [1, 2)
  const int64_t half = tot >= 0 ? tot / 2 : -((-tot + 1) / 2);
  const double mc = (tot - 2 * half) ? 2.0 * m : m;
  Flt y = flt_from_f64(1.0 / std::sqrt(mc), 64);
  y.exp -= half;
  const Flt one = flt_from_u64(1, 64);
  uint64_t cur = 48;
  while (cur < target) {
    cur = std::min(2 * cur, target);
    const uint64_t w = cur + 32;
    Flt xt = truncated_to_prec(self, w);
    Flt y2 = mul_at_prec(y, y, w);
    Flt er = sub_at_prec(one, mul_at_prec(xt, y2, w), w);  // |er| ~ 2^-(cur/2)
    er = truncated_to_prec(er, cur / 2 + 64);
    Flt c = mul_at_prec(y, er, w);
    c.exp -= 1;
    y = add_at_prec(y, c, w);
  }
  self = mul_at_prec(self, y, prec);
}

static Flt pow_int(const Flt& base0, const Int& ex) {  // float.rs:246-270
  uint64_t prec = base0.prec;
  Flt result = flt_from_u64(1, prec);
  if (ex.zero()) return result;
  Flt base = base0;
  uint64_t nb = bits_of(ex.m);
  for (uint64_t i = 0; i < nb; i++) {
    if (bit_at(ex.m, i)) result = mul_at_prec(result, base, prec);
    if (i + 1 < nb) base = mul_at_prec(base, base, prec);
  }
  return result;
}

static Int to_integer_down(const Flt& f) {  // float.rs:199-241 (non-negative use)
  if (f.zero()) return Int();
  if (f.exp >= 0) return Int(f.exp ? shl_mag(f.mant, (uint64_t)f.exp) : f.mant, f.sign);
  uint64_t s = (uint64_t)(-f.exp);
  Limbs t = shr_mag(f.mant, s);
  bool low = has_low_bits(f.mant, s);
  Int r(t, false);
  if (f.sign && (!r.zero() || low)) {
    if (low) r = add(r, Int(1));
    r.neg = !r.zero();
  }
  return r;
}

// ------------------------------------------------------------------ division
static void divrem(const Int& a, const Int& b, Int& q, Int& r);

static void divrem_newton(const Int& a, const Int& b, Int& q, Int& r) {  // integer.rs:1031-1083
  uint64_t ab = bits_of(a.m), bb = bits_of(b.m);
  uint64_t qb = ab - bb + 1, prec = qb + 64;
  Flt recip = reciprocal_at_prec(flt_from_int(b), prec);
  Flt at = truncated_to_prec(flt_from_int(a), prec);
  Flt qf = mul_at_prec(at, recip, prec);
  q = to_integer_down(qf);
  r = sub(a, mul(q, b));
  while (r.neg && !r.zero()) {
    q = sub(q, Int(1));
    r = add(r, b);
  }
  while (!r.neg && cmp_mag(r.m, b.m) >= 0) {
    q = add(q, Int(1));
    r = sub(r, b);
  }
}

static void divrem(const Int& a, const Int& b, Int& q, Int& r) {  // integer.rs:1004-1029
  if (b.m.size() >= g_newton_div_threshold && a.m.size() >= g_newton_div_threshold && cmp_mag(a.m, b.m) >= 0) {
    divrem_newton(a, b, q, r);
    return;
  }
  Limbs ql, rl;
  divrem_knuth(a.m, b.m, ql, rl);
  q = Int(ql, false);
  r = Int(rl, false);
}

static Int pow_u(uint64_t base, uint64_t e) {  // integer.rs:68-82
  Int result(1), b(base);
  while (e) {
    if (e & 1) result = mul(result, b);
    e >>= 1;
    if (e) b = mul(b, b);
  }
  return result;
}

// ------------------------------------------------------------------ decimal
static const uint64_t DEC_CHUNK = 10000000000000000000ull;  // 10^19 (integer.rs:887-888)

// (u1:u0) / d for the invariant d = 10^19 (bit 63 set) and u1 < d, with the
// precomputed reciprocal v = floor((2^128 - 1) / d) - 2^64 (Moller and
// Granlund, "Improved division by invariant integers", 2011, Algorithm 4).
static const uint64_t DEC_CHUNK_INV = (uint64_t)((~(u128)0) / DEC_CHUNK - ((u128)1 << 64));
static inline uint64_t div_dec_chunk(uint64_t u1, uint64_t u0, uint64_t& r) {
  u128 q = (u128)DEC_CHUNK_INV * u1;
  q += ((u128)(u1 + 1) << 64) | u0;
  uint64_t q1 = (uint64_t)(q >> 64), q0 = (uint64_t)q;
  uint64_t rr = u0 - q1 * DEC_CHUNK;
  if (rr > q0) {
    q1--;
    rr += DEC_CHUNK;
  }
  if (rr >= DEC_CHUNK) {
    q1++;
    rr -= DEC_CHUNK;
  }
  r = rr;
  return q1;
}

static std::string decimal_naive(Limbs mag) {  // integer.rs:968-983
  std::vector<uint64_t> chunks;
  while (!mag.empty()) {
    uint64_t rem = 0;
    for (size_t i = mag.size(); i-- > 0;) mag[i] = div_dec_chunk(rem, mag[i], rem);
    trim(mag);
    chunks.push_back(rem);
  }
  std::string out = std::to_string(chunks.back());
  char buf[32];
  for (size_t i = chunks.size() - 1; i-- > 0;) {
    snprintf(buf, sizeof buf, "%019llu", (unsigned long long)chunks[i]);
    out += buf;
  }
  return out;
}

static uint64_t dec_estimate(uint64_t bits) { return (uint64_t)std::ceil((double)bits * 0.301029995663981); }

static std::string to_decimal_padded(const Int& n, size_t want);

static std::string to_decimal_top(const Int& n) {  // integer.rs:892-930
  if (n.m.size() <= g_to_string_dc_threshold) return decimal_naive(n.m);
  uint64_t m = dec_estimate(bits_of(n.m)) / 2;
  if (m == 0) return decimal_naive(n.m);
  Int sp = pow_u(10, m), hi, lo;
  divrem(n, sp, hi, lo);
  std::string hs, ls;
  if (n.m.size() >= 4096) {
    Worker t([&] { ls = to_decimal_padded(lo, m); });
    hs = to_decimal_top(hi);
    t.join();
  } else {
    hs = to_decimal_top(hi);
    ls = to_decimal_padded(lo, m);
  }
  return hs + ls;
}

static std::string to_decimal_padded(const Int& n, size_t want) {  // integer.rs:932-964
  if (n.zero()) return std::string(want, '0');
  if (n.m.size() <= g_to_string_dc_threshold) {
    std::string s = decimal_naive(n.m);
    return std::string(want - s.size(), '0') + s;
  }
  size_t m = want / 2;
  Int sp = pow_u(10, m), hi, lo;
  divrem(n, sp, hi, lo);
  std::string hs, ls;
  if (n.m.size() >= 4096) {
    Worker t([&] { ls = to_decimal_padded(lo, m); });
    hs = to_decimal_padded(hi, want - m);
    t.join();
  } else {
    hs = to_decimal_padded(hi, want - m);
    ls = to_decimal_padded(lo, m);
  }
  return hs + ls;
}

// ------------------------------------------------------------------ Chudnovsky
static const uint64_t CH_A = 13591409, CH_B = 545140134;  // chudnovsky.rs:57-58
static const uint64_t C3_OVER_24 = 10939058860032000ull;  // chudnovsky.rs:61
static const double DIGITS_PER_TERM = 14.181647462725478;  // chudnovsky.rs:50
static const uint64_t SAFETY_TERMS = 8;                    // chudnovsky.rs:55

struct PQT {
  Int p, q, t;
};

// ------------------------------------------------------- small-range splitting
// The same (P, Q, T) as the recursion below for a range of at most
// LEAF_MAX terms, without heap traffic: terms from u128 arithmetic, then
// neighbouring pairs merged level by level in two flat per-thread buffers
// (schoolbook products; the merge is associative, so the bracketing does
// not change the result).
static const uint64_t LEAF_MAX = 128;

struct RawNode {
  uint32_t po, qo, to;  // offsets of |P|, |Q|, |T| in the level buffer
  uint32_t pn, qn, tn;  // lengths in limbs (trimmed)
  bool ps, ts;          // signs of P and T (Q > 0)
};

static uint32_t raw_trim(const uint64_t* x, uint32_t n) {
  while (n && x[n - 1] == 0) n--;
  return n;
}

static uint32_t raw_mul(const uint64_t* x, uint32_t nx, const uint64_t* y, uint32_t ny, uint64_t* z) {
  if (!nx || !ny) return 0;
  memset(z, 0, (nx + ny) * 8);
  for (uint32_t i = 0; i < nx; i++) {
    u128 carry = 0;
    const uint64_t xi = x[i];
    for (uint32_t j = 0; j < ny; j++) {
      u128 cur = (u128)z[i + j] + (u128)xi * y[j] + carry;
      z[i + j] = (uint64_t)cur;
      carry = cur >> 64;
    }
    z[i + ny] = (uint64_t)carry;
  }
  return raw_trim(z, nx + ny);
}

static int raw_cmp(const uint64_t* x, uint32_t nx, const uint64_t* y, uint32_t ny) {
  if (nx != ny) return nx < ny ? -1 : 1;
  for (uint32_t i = nx; i-- > 0;)
    if (x[i] != y[i]) return x[i] < y[i] ? -1 : 1;
  return 0;
}

// z = (sx ? -|x| : |x|) + (sy ? -|y| : |y|); returns |z|'s length, sign in sz.
static uint32_t raw_add_signed(const uint64_t* x, uint32_t nx, bool sx, const uint64_t* y, uint32_t ny, bool sy,
                               uint64_t* z, bool& sz) {
  if (sx == sy) {
    if (nx < ny) {
      std::swap(x, y);
      std::swap(nx, ny);
    }
    u128 c = 0;
    for (uint32_t i = 0; i < nx; i++) {
      c += (u128)x[i] + (i < ny ? y[i] : 0);
      z[i] = (uint64_t)c;
      c >>= 64;
    }
    z[nx] = (uint64_t)c;
    sz = sx;
    return raw_trim(z, nx + 1);
  }
  int c = raw_cmp(x, nx, y, ny);
  if (c == 0) {
    sz = false;
    return 0;
  }
  if (c < 0) {
    std::swap(x, y);
    std::swap(nx, ny);
    std::swap(sx, sy);
  }
  uint64_t borrow = 0;
  for (uint32_t i = 0; i < nx; i++) {
    uint64_t yi = i < ny ? y[i] : 0;
    uint64_t d = x[i] - yi - borrow;
    borrow = (x[i] < yi || (x[i] == yi && borrow)) ? 1 : 0;
    z[i] = d;
  }
  sz = sx;
  return raw_trim(z, nx);
}

static PQT split_leaf(uint64_t a, uint64_t b) {
  const uint32_t m = (uint32_t)(b - a);
  thread_local std::vector<uint64_t> buf0, buf1, tq, pt;
  const size_t cap = 64 * (size_t)m + 256;  // a level holds about 12 limbs per term
  if (buf0.size() < cap) {
    buf0.resize(cap);
    buf1.resize(cap);
    tq.resize(cap);
    pt.resize(cap);
  }
  std::vector<RawNode> nodes(m), next;
  uint64_t* cur = buf0.data();
  uint64_t* nxt = buf1.data();
  uint32_t off = 0;
  for (uint32_t i = 0; i < m; i++) {
    const uint64_t k = a + i;
    // p = -(6k-5)(2k-1)(6k-1), q = (C^3/24) k^3, t = p (A + B k)   (chudnovsky.rs:377-390)
    u128 pm = (u128)(6 * k - 5) * (2 * k - 1);
    uint64_t p3[3], f[1] = {6 * k - 1};
    uint64_t pl[2] = {(uint64_t)pm, (uint64_t)(pm >> 64)};
    uint32_t pn = raw_mul(pl, raw_trim(pl, 2), f, 1, p3);
    u128 k2 = (u128)k * k;
    uint64_t k2l[2] = {(uint64_t)k2, (uint64_t)(k2 >> 64)}, kk[1] = {k}, k3[3], c3[1] = {C3_OVER_24}, q4[4];
    uint32_t k3n = raw_mul(k2l, raw_trim(k2l, 2), kk, 1, k3);
    uint32_t qn = raw_mul(k3, k3n, c3, 1, q4);
    u128 ab = (u128)CH_A + (u128)CH_B * k;
    uint64_t abl[2] = {(uint64_t)ab, (uint64_t)(ab >> 64)}, t5[5];
    uint32_t tn = raw_mul(p3, pn, abl, raw_trim(abl, 2), t5);
    RawNode& n = nodes[i];
    n.po = off, n.pn = pn, memcpy(cur + off, p3, pn * 8), off += pn;
    n.qo = off, n.qn = qn, memcpy(cur + off, q4, qn * 8), off += qn;
    n.to = off, n.tn = tn, memcpy(cur + off, t5, tn * 8), off += tn;
    n.ps = true;
    n.ts = true;
  }
  while (nodes.size() > 1) {
    const size_t np = nodes.size() / 2;
    next.resize(np + (nodes.size() & 1));
    uint32_t o = 0;
    for (size_t i = 0; i < np; i++) {
      const RawNode& L = nodes[2 * i];
      const RawNode& R = nodes[2 * i + 1];
      RawNode z;
      z.po = o;
      z.pn = raw_mul(cur + L.po, L.pn, cur + R.po, R.pn, nxt + o);
      z.ps = L.ps != R.ps;
      o += z.pn;
      z.qo = o;
      z.qn = raw_mul(cur + L.qo, L.qn, cur + R.qo, R.qn, nxt + o);
      o += z.qn;
      uint32_t a1 = raw_mul(cur + L.to, L.tn, cur + R.qo, R.qn, tq.data());
      uint32_t a2 = raw_mul(cur + L.po, L.pn, cur + R.to, R.tn, pt.data());
      z.to = o;
      z.tn = raw_add_signed(tq.data(), a1, L.ts, pt.data(), a2, L.ps != R.ts, nxt + o, z.ts);
      o += z.tn;
      next[i] = z;
    }
    if (nodes.size() & 1) {
      const RawNode& L = nodes.back();
      RawNode z = L;
      z.po = o, memcpy(nxt + o, cur + L.po, L.pn * 8), o += L.pn;
      z.qo = o, memcpy(nxt + o, cur + L.qo, L.qn * 8), o += L.qn;
      z.to = o, memcpy(nxt + o, cur + L.to, L.tn * 8), o += L.tn;
      next[np] = z;
    }
    nodes.swap(next);
    std::swap(cur, nxt);
  }
  const RawNode& r = nodes[0];
  PQT out;
  out.p = Int(Limbs(cur + r.po, cur + r.po + r.pn), r.ps);
  out.q = Int(Limbs(cur + r.qo, cur + r.qo + r.qn), false);
  out.t = Int(Limbs(cur + r.to, cur + r.to + r.tn), r.ts);
  return out;
}

// chudnovsky.rs:377-413 (rayon::join on subtrees of >= 64 terms becomes a
// host thread for the top levels); ranges of at most LEAF_MAX terms take
// the flat path above.
static PQT split(uint64_t a, uint64_t b, int depth) {
  if (b - a <= LEAF_MAX && a >= 1) return split_leaf(a, b);
  if (b - a == 1) {
    Int k(a);
    Int f1 = sub(mulu(k, 6), Int(5)), f2 = sub(mulu(k, 6), Int(1)), f3 = sub(mulu(k, 2), Int(1));
    Int p = neg(mul(mul(f1, f2), f3));
    Int q = mul(Int(C3_OVER_24), mul(mul(k, k), k));
    Int t = mul(p, add(Int(CH_A), mulu(k, CH_B)));
    return PQT{p, q, t};
  }
  uint64_t m = (a + b) / 2;
  PQT L, R;
  if (b - a >= PARALLEL_SPLIT && depth < 4) {
    Worker th([&] { R = split(m, b, depth + 1); });
    L = split(a, m, depth + 1);
    th.join();
  } else {
    L = split(a, m, depth);
    R = split(m, b, depth);
  }
  PQT o;
  o.t = add(mul(L.t, R.q), mul(L.p, R.t));
  o.p = mul(L.p, R.p);
  o.q = mul(L.q, R.q);
  return o;
}

// Root without P (chudnovsky.rs:339-369).
static void split_root(uint64_t a, uint64_t b, Int& q, Int& t) {
  if (b - a == 1) {
    PQT x = split(a, b, 0);
    q = x.q;
    t = x.t;
    return;
  }
  uint64_t m = (a + b) / 2;
  PQT L, R;
  Worker th([&] { R = split(m, b, 1); });
  L = split(a, m, 1);
  th.join();
  t = add(mul(L.t, R.q), mul(L.p, R.t));
  q = mul(L.q, R.q);
}

static double now_ms() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Float from an f64 at prec (Float::with_val_64(prec, f64)).
static Flt flt_f64_prec(double v, uint64_t prec) {
  Flt f = flt_from_f64(v, 64);
  f.prec = prec;
  round_to_prec(f);
  return f;
}

// Gauss-Legendre AGM (crates/pi-core/src/algorithm/gauss_legendre.rs:61-151):
// iterations = ceil(log2 prec) + 2; per iteration a' = (a+b)/2,
// b' = sqrt(a b), t -= p (a - a')^2, p <<= 1; pi = (a+b)^2 / t / 4.
static Flt gauss_legendre(uint64_t prec, bool fast_sqrt) {
  auto root = [&](Flt& x) {
    if (fast_sqrt) sqrt_fast(x);
    else sqrt_mut(x);
  };
  const uint32_t iters = (uint32_t)std::ceil(std::log2((double)prec)) + 2;
  Flt a = flt_from_u64(1, prec);
  Flt b = flt_f64_prec(0.5, prec);
  root(b);
  Flt t = flt_f64_prec(0.25, prec);
  Int p(1);
  for (uint32_t it = 0; it < iters; it++) {
    Flt an = add_at_prec(a, b, prec);
    an = div_at_prec(an, flt_from_u64(2, 64), prec);
    Flt bn = mul_at_prec(a, b, prec);
    root(bn);
    Flt diff = sub_at_prec(a, an, prec);
    Flt dsq = mul_at_prec(diff, diff, prec);
    dsq = mul_at_prec(dsq, flt_from_int(p), prec);
    t = sub_at_prec(t, dsq, prec);
    a = an;
    b = bn;
    p = Int(shl_mag(p.m, 1), false);
  }
  Flt pi = add_at_prec(a, b, prec);
  Flt sq = pi;  // square_mut: mantissa^2, exp doubled, rounded to prec
  sq.mant = mul_mag(pi.mant, pi.mant);
  sq.exp = 2 * pi.exp;
  sq.sign = false;
  round_to_prec(sq);
  sq = div_at_prec(sq, t, prec);
  return div_at_prec(sq, flt_from_u64(4, 64), prec);
}

// ------------------------------------------------- batched binary splitting
// Level-synchronous form of the binary splitting above (the device-batched
// drive of chudnovsky.rs:377-413): leaves of `leaf` terms are split on host
// threads, then every level merges neighbouring pairs,
//   P = P_L P_R,   Q = Q_L Q_R,   T = T_L Q_R + P_L T_R,
// with all of the level's products in one pimul_mul_batch call (operands
// staged through one pinned buffer, one copy each way) and T's sum on host
// threads.  The merge is associative, so the root (Q, T) is exactly the
// recursive split's, whatever the bracketing.

static void parallel_for(size_t n, const std::function<void(size_t, size_t)>& fn) {
  const size_t nt = std::max(1u, std::thread::hardware_concurrency());
  if (n <= 1 || nt == 1) {
    fn(0, n);
    return;
  }
  const size_t parts = std::min(n, nt);
  const size_t per = (n + parts - 1) / parts;
  std::list<Worker> th;  // Workers do not move: a list constructs them in place
  for (size_t i = 1; i < parts; i++) {
    size_t lo = i * per, hi = std::min(n, lo + per);
    if (lo < hi) th.emplace_back([&fn, lo, hi] { fn(lo, hi); });
  }
  fn(0, std::min(n, per));
  std::exception_ptr first;
  for (auto& t : th) {
    try {
      t.join();
    } catch (...) {
      if (!first) first = std::current_exception();
    }
  }
  if (first) std::rethrow_exception(first);
}

// Pinned host staging, a device buffer and a stream, grown on demand.
struct LevelStaging {
  cudaStream_t st = nullptr;
  uint64_t* h = nullptr;
  size_t h_words = 0;
  uint64_t* d = nullptr;
  size_t d_words = 0;
  ~LevelStaging() {
    if (h) cudaFreeHost(h);
    if (d) cudaFree(d);
    if (st) cudaStreamDestroy(st);
  }
  int init() {
    if (!st && cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return PIMUL_ECUDA;
    return PIMUL_OK;
  }
  int host(size_t w) {
    if (w <= h_words) return PIMUL_OK;
    if (h) cudaFreeHost(h);
    h = nullptr;
    size_t n = std::max(w, h_words + h_words / 2);
    if (cudaHostAlloc((void**)&h, std::max<size_t>(n, 1) * 8, cudaHostAllocDefault) != cudaSuccess) {
      h_words = 0;
      return PIMUL_ENOMEM;
    }
    h_words = n;
    return PIMUL_OK;
  }
  int dev(size_t w) {
    if (w <= d_words) return PIMUL_OK;
    if (d) cudaFree(d);
    d = nullptr;
    size_t n = std::max(w, d_words + d_words / 2);
    if (cudaMalloc((void**)&d, std::max<size_t>(n, 1) * 8) != cudaSuccess) {
      d_words = 0;
      return PIMUL_ENOMEM;
    }
    d_words = n;
    return PIMUL_OK;
  }
};

// Wall-time split of the batched drivers (ms): host staging, GPU round trip
// (copies + batch), host unpacking, host-side products, node combine.

// Products a[i] * b[i] of magnitudes.  Those whose smaller operand has at
// least gpu_min limbs go to the GPU in one pimul_mul_batch call: operands
// deduplicated by address and staged through one pinned buffer (one copy
// each way); the rest run on host threads through mul_mag.
static int batch_mul(const std::vector<const Limbs*>& A, const std::vector<const Limbs*>& B,
                     std::vector<Limbs>& out, LevelStaging& S, size_t gpu_min) {
  const size_t n = A.size();
  out.assign(n, Limbs());
  std::vector<size_t> gi, ci;
  for (size_t i = 0; i < n; i++) {
    size_t la = A[i]->size(), lb = B[i]->size();
    if (!la || !lb) continue;
    bool fits = 4 * (la + lb) <= (1ull << 32);
    (fits && std::min(la, lb) >= gpu_min ? gi : ci).push_back(i);
  }
  if (!gi.empty()) {
    std::unordered_map<const Limbs*, size_t> off;
    std::vector<const Limbs*> uniq;
    std::vector<size_t> uoff, ooff(gi.size() + 1);
    size_t in_w = 0, out_w = 0;
    for (size_t g = 0; g < gi.size(); g++) {
      for (const Limbs* x : {A[gi[g]], B[gi[g]]}) {
        if (off.emplace(x, in_w).second) {
          uniq.push_back(x);
          uoff.push_back(in_w);
          in_w += x->size();
        }
      }
      ooff[g] = out_w;
      out_w += A[gi[g]]->size() + B[gi[g]]->size();
    }
    ooff[gi.size()] = out_w;
    double t0 = now_ms();
    int rc = S.host(std::max(in_w, out_w));
    if (!rc) rc = S.dev(in_w + out_w);
    if (rc) return rc;
    parallel_for(uniq.size(), [&](size_t lo, size_t hi) {
      for (size_t u = lo; u < hi; u++) memcpy(S.h + uoff[u], uniq[u]->data(), uniq[u]->size() * 8);
    });
    uint64_t* d_in = S.d;
    uint64_t* d_out = S.d + in_w;
    std::vector<pimul_job> jobs(gi.size());
    for (size_t g = 0; g < gi.size(); g++) {
      const Limbs* a = A[gi[g]];
      const Limbs* b = B[gi[g]];
      jobs[g] = pimul_job{d_in + off[a], a->size(), d_in + off[b], b->size(), d_out + ooff[g]};
      uint64_t L2 = 0;
      while ((1ull << L2) < 4 * (a->size() + b->size()) - 1) L2++;
      C().ntt_hist[L2].fetch_add(1, std::memory_order_relaxed);
    }
    C().ntt_calls.fetch_add(gi.size(), std::memory_order_relaxed);
    double t1 = now_ms();
    if (cudaMemcpyAsync(d_in, S.h, in_w * 8, cudaMemcpyHostToDevice, S.st) != cudaSuccess) return PIMUL_ECUDA;
    rc = pimul_mul_batch(jobs.data(), jobs.size(), S.st);
    if (rc) return rc;
    if (cudaMemcpyAsync(S.h, d_out, out_w * 8, cudaMemcpyDeviceToHost, S.st) != cudaSuccess) return PIMUL_ECUDA;
    if (cudaStreamSynchronize(S.st) != cudaSuccess) return PIMUL_ECUDA;
    double t2 = now_ms();
    parallel_for(gi.size(), [&](size_t lo, size_t hi) {
      for (size_t g = lo; g < hi; g++) {
        Limbs r(S.h + ooff[g], S.h + ooff[g + 1]);
        trim(r);
        out[gi[g]] = std::move(r);
      }
    });
    double t3 = now_ms();
    bt_add(0, t1 - t0);
    bt_add(1, t2 - t1);
    bt_add(2, t3 - t2);
  }
  double t4 = now_ms();
  parallel_for(ci.size(), [&](size_t lo, size_t hi) {
    for (size_t c = lo; c < hi; c++) out[ci[c]] = mul_mag(*A[ci[c]], *B[ci[c]]);
  });
  bt_add(3, now_ms() - t4);
  return C().error.load();
}

// One level: nodes[2i], nodes[2i+1] -> next[i]; an odd last node moves up as
// it is.  At the root level (one pair) P is not needed.
static int merge_level(std::vector<PQT>& nodes, LevelStaging& S) {
  const size_t np = nodes.size() / 2;
  const bool need_p = nodes.size() > 2;
  const int per = need_p ? 4 : 3;
  std::vector<const Limbs*> A, B;
  A.reserve(np * per);
  B.reserve(np * per);
  for (size_t i = 0; i < np; i++) {
    const PQT& L = nodes[2 * i];
    const PQT& R = nodes[2 * i + 1];
    A.push_back(&L.t.m), B.push_back(&R.q.m);  // T_L Q_R
    A.push_back(&L.p.m), B.push_back(&R.t.m);  // P_L T_R
    A.push_back(&L.q.m), B.push_back(&R.q.m);  // Q_L Q_R
    if (need_p) A.push_back(&L.p.m), B.push_back(&R.p.m);  // P_L P_R
  }
  std::vector<Limbs> prod;
  int rc = batch_mul(A, B, prod, S, 1);
  if (rc) return rc;
  double t0 = now_ms();
  std::vector<PQT> next(np + (nodes.size() & 1));
  parallel_for(np, [&](size_t lo, size_t hi) {
    for (size_t i = lo; i < hi; i++) {
      const PQT& L = nodes[2 * i];
      const PQT& R = nodes[2 * i + 1];
      Limbs* pr = &prod[per * i];
      PQT o;
      o.t = add(Int(std::move(pr[0]), L.t.neg), Int(std::move(pr[1]), L.p.neg != R.t.neg));
      o.q = Int(std::move(pr[2]), false);
      if (need_p) o.p = Int(std::move(pr[3]), L.p.neg != R.p.neg);
      next[i] = std::move(o);
    }
  });
  if (nodes.size() & 1) next[np] = std::move(nodes.back());
  nodes.swap(next);
  bt_add(4, now_ms() - t0);
  C().batch_levels.fetch_add(1, std::memory_order_relaxed);
  return PIMUL_OK;
}


static void report_split(const char* what) {
  if (!getenv("PIMUL_PI_TIMING")) return;
  fprintf(stderr, "[pimul] %s: leaves %.1f ms, staging %.1f, gpu %.1f, unpack %.1f, host products %.1f, "
          "bookkeeping %.1f\n", what, C().leaf_ms, C().bt[0], C().bt[1], C().bt[2], C().bt[3], C().bt[4]);
  for (double& x : C().bt) x = 0;
  C().leaf_ms = 0;
}

// ---------------------------------------------- device-resident splitting
// The levels above the leaves without host round trips: the leaves' P, Q, T
// are uploaded once, and every level's products (pimul_mul_batch), T sums
// (pimul_addsub_batch) and trimmed lengths (pimul_top_limbs) run on the
// device; only the root's Q and T come back.  Signs are static: every
// p_k < 0, so P of m terms has sign (-1)^m, and T < 0 for every range
// because its first term outweighs the rest (|p_k / q_k| < 10^-14), so
// |T| = |T_L| Q_R + (-1)^(m_L) |P_L| |T_R| is a sum or a difference of
// magnitudes (a borrow out of the top would be reported, never silent).
struct DNode {
  uint64_t* p;
  uint64_t* q;
  uint64_t* t;
  size_t pn, qn, tn;
  uint64_t terms;
};

// Nodes on the device and the arenas that hold them.
struct DLevel {
  std::vector<DNode> nodes;
  std::vector<uint64_t*> arenas;
};

static void dev_free(DLevel& L, cudaStream_t st) {
  for (uint64_t* a : L.arenas) cudaFreeAsync(a, st);
  L.arenas.clear();
  L.nodes.clear();
}

// The level products' batch option: long products that would half fill
// their transform run as wrapped cyclic products (PIMUL_BATCH_WRAP);
// PIMUL_PI_WRAP=0 turns it off.
static unsigned wrap_flags() {
  const char* e = getenv("PIMUL_PI_WRAP");
  return (!e || atoi(e) != 0) ? PIMUL_BATCH_WRAP : 0u;
}

// Levels until one node is left; keep_p keeps P of the last node (needed
// when it is merged again later).
static int dev_reduce(DLevel& Lv, cudaStream_t st, bool keep_p, size_t stop = 1) {
  int rc = PIMUL_OK;
  auto cu = [&](cudaError_t e) {
    if (e != cudaSuccess && !rc) rc = PIMUL_ECUDA;
    return e == cudaSuccess;
  };
  std::vector<DNode>& nodes = Lv.nodes;
  while (!rc && nodes.size() > stop) {
    double t0 = now_ms();
    const size_t np = nodes.size() / 2;
    const bool need_p = nodes.size() > 2 || keep_p, odd = nodes.size() & 1;
    // new level: Q, P, T per pair (and the odd node).  T = T_L Q_R + P_L T_R
    // is one fused sum (its spectra added before one inverse transform);
    // a difference goes through the temporaries T_L Q_R, P_L T_R and a
    // batched subtraction.  Q_L Q_R and T_L Q_R share Q_R's spectrum, and
    // P_R P_L and T_R P_L share P_L's (the batch shares the second factor's
    // spectrum among products of one transform length).
    size_t lvl_w = 0, tmp_w = 0;
    for (size_t i = 0; i < np; i++) {
      const DNode& L = nodes[2 * i];
      const DNode& R = nodes[2 * i + 1];
      lvl_w += L.qn + R.qn + (need_p ? L.pn + R.pn : 0) + std::max(L.tn + R.qn, L.pn + R.tn) + 1;
      if (L.terms & 1) tmp_w += L.tn + R.qn + L.pn + R.tn;
    }
    if (odd) lvl_w += nodes.back().pn + nodes.back().qn + nodes.back().tn;
    uint64_t* nxt = nullptr;
    uint64_t* tmp = nullptr;
    if (!cu(cudaMallocAsync((void**)&nxt, lvl_w * 8, st))) break;
    if (tmp_w && !cu(cudaMallocAsync((void**)&tmp, tmp_w * 8, st))) {
      cudaFreeAsync(nxt, st);
      break;
    }
    std::vector<DNode> next(np + odd);
    std::vector<pimul_sum_job> sj;
    std::vector<pimul_addsub_job> aj;
    sj.reserve(np * 3);
    size_t nprod = 0;
    uint64_t hist[33] = {0};
    auto count = [&](size_t la, size_t lb) {
      hist[64 - __builtin_clzll(4 * (la + lb) - 2)]++;  // ceil(log2(4 (la + lb) - 1))
      nprod++;
    };
    size_t lo = 0, to = 0;
    for (size_t i = 0; i < np; i++) {
      const DNode& L = nodes[2 * i];
      const DNode& R = nodes[2 * i + 1];
      DNode& z = next[i];
      z.terms = L.terms + R.terms;
      z.q = nxt + lo, z.qn = L.qn + R.qn, lo += z.qn;
      sj.push_back(pimul_sum_job{L.q, L.qn, R.q, R.qn, nullptr, 0, nullptr, 0, z.q, z.qn});
      count(L.qn, R.qn);
      if (need_p) {
        z.p = nxt + lo, z.pn = L.pn + R.pn, lo += z.pn;
        sj.push_back(pimul_sum_job{R.p, R.pn, L.p, L.pn, nullptr, 0, nullptr, 0, z.p, z.pn});
        count(L.pn, R.pn);
      } else {
        z.p = nullptr, z.pn = 0;
      }
      z.tn = std::max(L.tn + R.qn, L.pn + R.tn) + 1;
      z.t = nxt + lo, lo += z.tn;
      count(L.tn, R.qn);
      count(L.pn, R.tn);
      if (!(L.terms & 1)) {
        sj.push_back(pimul_sum_job{L.t, L.tn, R.q, R.qn, R.t, R.tn, L.p, L.pn, z.t, z.tn});
      } else {
        uint64_t* tq = tmp + to;
        to += L.tn + R.qn;
        uint64_t* pt = tmp + to;
        to += L.pn + R.tn;
        sj.push_back(pimul_sum_job{L.t, L.tn, R.q, R.qn, nullptr, 0, nullptr, 0, tq, L.tn + R.qn});
        sj.push_back(pimul_sum_job{R.t, R.tn, L.p, L.pn, nullptr, 0, nullptr, 0, pt, L.pn + R.tn});
        aj.push_back(pimul_addsub_job{tq, L.tn + R.qn, pt, L.pn + R.tn, z.t, z.tn, 1});
      }
    }
    if (odd) {
      const DNode& o = nodes.back();
      DNode& z = next[np];
      z = o;
      z.p = nxt + lo, lo += o.pn;
      z.q = nxt + lo, lo += o.qn;
      z.t = nxt + lo, lo += o.tn;
      cu(cudaMemcpyAsync(z.p, o.p, o.pn * 8, cudaMemcpyDeviceToDevice, st));
      cu(cudaMemcpyAsync(z.q, o.q, o.qn * 8, cudaMemcpyDeviceToDevice, st));
      cu(cudaMemcpyAsync(z.t, o.t, o.tn * 8, cudaMemcpyDeviceToDevice, st));
    }
    C().ntt_calls.fetch_add(nprod, std::memory_order_relaxed);
    for (int L2 = 0; L2 < 33; L2++)
      if (hist[L2]) C().ntt_hist[L2].fetch_add(hist[L2], std::memory_order_relaxed);
    double t1 = now_ms();
    if (!rc) rc = pimul_sum_batch_ex(sj.data(), sj.size(), st, wrap_flags());
    const double t_sum = now_ms();
    if (!rc && !aj.empty()) rc = pimul_addsub_batch(aj.data(), aj.size(), st);
    const double t_as = now_ms();
    if (tmp) cudaFreeAsync(tmp, st);
    for (uint64_t* a : Lv.arenas) cudaFreeAsync(a, st);
    Lv.arenas.assign(1, nxt);
    // trimmed lengths of the new level
    std::vector<const uint64_t*> arrs;
    std::vector<size_t> lens;
    arrs.reserve(next.size() * 3);
    for (const DNode& z : next) {
      if (z.pn) arrs.push_back(z.p), lens.push_back(z.pn);
      arrs.push_back(z.q), lens.push_back(z.qn);
      arrs.push_back(z.t), lens.push_back(z.tn);
    }
    std::vector<size_t> got(arrs.size());
    const double t_arr = now_ms();
    if (!rc) rc = pimul_top_limbs(arrs.data(), lens.data(), arrs.size(), got.data(), st);
    double t2 = now_ms();
    if (!rc) {
      size_t k = 0;
      for (DNode& z : next) {
        if (z.pn) z.pn = got[k++];
        z.qn = got[k++];
        z.tn = got[k++];
      }
    }
    if (getenv("PIMUL_PI_TIMING") && !next.empty())
      fprintf(stderr, "[pimul]   level: %zu pairs, %zu products, top Q %zu limbs, %.1f ms (build %.1f, sum call %.1f, "
              "subtract %.1f, lengths %.1f + %.1f)\n", np, nprod, next[0].qn, t2 - t1, t1 - t0, t_sum - t1,
              t_as - t_sum, t_arr - t_as, t2 - t_arr);
    nodes.swap(next);
    C().batch_levels.fetch_add(1, std::memory_order_relaxed);
    bt_add(1, t2 - t1);
    bt_add(4, (t1 - t0));
  }
  return rc;
}

// The root's Q and |T| left on the device for the final assembly; with
// top_limbs set (the number of top limbs of Q and of A Q + T the consumer
// reads) the root is Q_hi 2^(64 q_off), |T|_hi 2^(64 t_off), from operands
// cut to their top limbs.
struct DevRoot {
  DLevel lvl;
  uint64_t top_limbs = 0;
  uint64_t q_off = 0, t_off = 0;
  std::vector<uint64_t> svc_handles;  // the served tree's root handles (freed after the final assembly)
};

// ---------------------------------------------------- served splitting tree
// The upper levels of the splitting tree driven through the multiply service
// (pimul_submit) as the recursion unfolds, the way the reference's
// recursion issues them (crates/pi-core/src/algorithm/chudnovsky.rs:377-413):
// every node's |P|, Q, |T| is a handle, each merge is five chained requests
// (P_L P_R, Q_L Q_R, |T_L| Q_R, |P_L| |T_R|, and their sum or difference
// with the static signs of the level-batched form), and a node's handles are
// released as soon as its parent's requests are queued.  Nothing returns to
// the host between levels; the service batches whatever is ready.
struct HNode {
  uint64_t p = 0, q = 0, t = 0;
  uint64_t terms = 0;
};

static int svc_req(int op, uint64_t a, uint64_t b, uint64_t* out) {
  uint64_t tk = 0;
  C().served_requests++;
  return pimul_submit(op, a, b, out, &tk);
}

static int serve_tree(const std::vector<HNode>& v, size_t lo, size_t hi, bool need_p, HNode& out) {
  if (hi - lo == 1) {
    out = v[lo];
    return PIMUL_OK;
  }
  const size_t m = (lo + hi) / 2;
  HNode L, R;
  int rc = serve_tree(v, lo, m, true, L);  // P_L enters T
  if (!rc) rc = serve_tree(v, m, hi, need_p, R);
  if (rc) return rc;
  uint64_t t1 = 0, t2 = 0;
  if (need_p) rc = svc_req(PIMUL_OP_MUL, L.p, R.p, &out.p);
  if (!rc) rc = svc_req(PIMUL_OP_MUL, L.q, R.q, &out.q);
  if (!rc) rc = svc_req(PIMUL_OP_MUL, L.t, R.q, &t1);
  if (!rc) rc = svc_req(PIMUL_OP_MUL, L.p, R.t, &t2);
  // |T| = |T_L| Q_R + (-1)^m_L |P_L| |T_R|  (P of m terms has sign (-1)^m, T < 0)
  if (!rc) rc = svc_req((L.terms & 1) ? PIMUL_OP_SUB : PIMUL_OP_ADD, t1, t2, &out.t);
  out.terms = L.terms + R.terms;
  for (uint64_t h : {t1, t2, L.p, L.q, L.t, R.p, R.q, R.t})
    if (h) pimul_release(h);
  return rc;
}

// Runs the served tree over the nodes of `top` (device arrays the caller
// keeps until the root is done) and puts the root's Q and |T| (trimmed) in
// keep->lvl as one node; their handles go to keep->svc_handles.
static int serve_root(const DLevel& top, cudaStream_t st, DevRoot* keep) {
  const double t0 = now_ms();
  if (cudaStreamSynchronize(st) != cudaSuccess) return PIMUL_ECUDA;  // the service streams read the nodes
  std::vector<HNode> v(top.nodes.size());
  int rc = PIMUL_OK;
  for (size_t i = 0; i < v.size() && !rc; i++) {
    const DNode& n = top.nodes[i];
    rc = pimul_adopt(n.p, n.pn, &v[i].p);
    if (!rc) rc = pimul_adopt(n.q, n.qn, &v[i].q);
    if (!rc) rc = pimul_adopt(n.t, n.tn, &v[i].t);
    v[i].terms = n.terms;
  }
  HNode root;
  const double t1 = now_ms();
  if (!rc) rc = serve_tree(v, 0, v.size(), false, root);
  if (rc) return rc;
  const double t2 = now_ms();
  const uint64_t* dq = nullptr;
  const uint64_t* dt = nullptr;
  size_t qn = 0, tn = 0;
  rc = pimul_handle_device(root.q, &dq, &qn);
  if (!rc) rc = pimul_handle_device(root.t, &dt, &tn);
  if (getenv("PIMUL_PI_TIMING"))
    fprintf(stderr, "[pimul] served tree: %zu nodes handed over (sync + adopt %.1f ms), requests queued in %.1f ms, "
            "root ready after %.1f ms\n", v.size(), t1 - t0, t2 - t1, now_ms() - t2);
  keep->svc_handles = {root.q, root.t};
  if (root.p) pimul_release(root.p);
  if (rc) return rc;
  const uint64_t* arrs[2] = {dq, dt};
  const size_t lens[2] = {qn, tn};
  size_t trimmed[2] = {0, 0};
  rc = pimul_top_limbs(arrs, lens, 2, trimmed, st);
  if (rc) return rc;
  DNode r{};
  r.q = const_cast<uint64_t*>(dq);
  r.t = const_cast<uint64_t*>(dt);
  r.qn = trimmed[0];
  r.tn = trimmed[1];
  r.terms = root.terms;
  keep->lvl.nodes = {r};
  keep->q_off = keep->t_off = 0;
  return PIMUL_OK;
}

// Root merge from the operands' top m + 2 limbs (m = top_limbs + 2): the
// cut parts move Q = Q_L Q_R and T = T_L Q_R +- P_L T_R by less than
// 2^-(64 m) relative (every dropped limb is below the kept m + 2 of its
// operand, and P_L T_R is the smaller term), and the products are about
// half as long: the root's 2^30-point transforms of a 10^9-digit run
// become 2^29-point ones.  T's two products drop the same total D of limbs
// so that their sum stays aligned; Q_R is cut the same way in Q and T
// (one shared spectrum).
static int dev_root_truncated(DLevel& Lv, cudaStream_t st, uint64_t top_limbs, DevRoot* keep) {
  const DNode& L = Lv.nodes[0];
  const DNode& R = Lv.nodes[1];
  const uint64_t m2 = top_limbs + 4;
  auto cut = [&](uint64_t n) { return n > m2 ? n - m2 : 0; };
  const uint64_t dxq = cut(L.qn), dyq = cut(R.qn), dx1 = cut(L.tn);
  const uint64_t D = dx1 + dyq;
  const uint64_t dy2 = std::min<uint64_t>(D, R.tn ? R.tn - 1 : 0), dx2 = D - dy2;
  if (!L.pn || !R.tn || !L.tn || dx2 + 1 > L.pn) return PIMUL_OK;  // leave the root to dev_reduce
  int rc = PIMUL_OK;
  const uint64_t qn = (L.qn - dxq) + (R.qn - dyq);
  const uint64_t n1 = (L.tn - dx1) + (R.qn - dyq), n2 = (L.pn - dx2) + (R.tn - dy2);
  const uint64_t tn = std::max(n1, n2) + 1;
  uint64_t* arena = nullptr;
  uint64_t* tmp = nullptr;
  const bool diff = (L.terms & 1) != 0;
  if (cudaMallocAsync((void**)&arena, (qn + tn) * 8, st) != cudaSuccess) return PIMUL_ENOMEM;
  if (diff && cudaMallocAsync((void**)&tmp, (n1 + n2) * 8, st) != cudaSuccess) {
    cudaFreeAsync(arena, st);
    return PIMUL_ENOMEM;
  }
  DNode z{};
  z.terms = L.terms + R.terms;
  z.q = arena, z.qn = qn;
  z.t = arena + qn, z.tn = tn;
  z.p = nullptr, z.pn = 0;
  std::vector<pimul_sum_job> sj;
  sj.push_back(pimul_sum_job{L.q + dxq, L.qn - dxq, R.q + dyq, R.qn - dyq, nullptr, 0, nullptr, 0, z.q, qn});
  if (!diff) {
    sj.push_back(pimul_sum_job{L.t + dx1, L.tn - dx1, R.q + dyq, R.qn - dyq, L.p + dx2, L.pn - dx2, R.t + dy2,
                               R.tn - dy2, z.t, tn});
  } else {
    sj.push_back(pimul_sum_job{L.t + dx1, L.tn - dx1, R.q + dyq, R.qn - dyq, nullptr, 0, nullptr, 0, tmp, n1});
    sj.push_back(pimul_sum_job{L.p + dx2, L.pn - dx2, R.t + dy2, R.tn - dy2, nullptr, 0, nullptr, 0, tmp + n1, n2});
  }
  C().ntt_calls.fetch_add(3, std::memory_order_relaxed);
  rc = pimul_sum_batch_ex(sj.data(), sj.size(), st, wrap_flags());
  if (!rc && diff) {
    pimul_addsub_job aj{tmp, n1, tmp + n1, n2, z.t, tn, 1};
    rc = pimul_addsub_batch(&aj, 1, st);
  }
  if (tmp) cudaFreeAsync(tmp, st);
  if (rc) {
    cudaFreeAsync(arena, st);
    return rc;
  }
  const uint64_t* arrs[2] = {z.q, z.t};
  size_t lens[2] = {z.qn, z.tn}, got[2] = {0, 0};
  rc = pimul_top_limbs(arrs, lens, 2, got, st);
  if (rc) {
    cudaFreeAsync(arena, st);
    return rc;
  }
  z.qn = got[0], z.tn = got[1];
  for (uint64_t* ar : Lv.arenas) cudaFreeAsync(ar, st);
  Lv.arenas.assign(1, arena);
  Lv.nodes.assign(1, z);
  keep->q_off = dxq + dyq;
  keep->t_off = D;
  return PIMUL_OK;
}

// Leaf size chosen per term range (pimul_pi_chudnovsky_batched with
// leaf_terms = 0).  A node of m terms near k has about m (3 log2 k +
// log2(C^3 / 24)) bits of Q, and every level doubles m, so the products of
// the first level (2 leaves, 2 m Q-bits in 16-bit coefficients) set the
// fill of every transform above it: runs of at most 4096 / (bits per term
// + 1) terms keep those products within 512 coefficients (and all higher
// ones within their power of two) instead of just over it.  The device
// leaves take two such runs (at most 64 terms).
static const uint64_t LEAF_AUTO = ~0ull;
static uint64_t auto_leaf(uint64_t k_hi) {
  const double bits = 3.0 * std::log2((double)std::max<uint64_t>(k_hi, 2)) + std::log2(10939058860032000.0) + 1.0;
  return std::max<uint64_t>(8, std::min<uint64_t>(32, (uint64_t)(4096.0 / bits)));
}

// The lowest levels of a segment merged by the one-CTA kernel (splitmerge.h),
// as one schedule captured in a CUDA graph: every level whose node pairs all
// need transforms of at most 2^12 points, stopping above `stop` nodes.  The
// leaves sit in fixed slots (sp, sq, st words); each merged level gets slots
// sized by the largest untrimmed product of the level, computed here from
// the leaves' exact lengths, and the trimmed lengths stay on the device until
// the last merged level, whose lengths are the only ones read back.  Lv
// becomes that level (its arena replaces the leaves').  Left nodes must hold
// an even number of terms (T a sum); otherwise, or when no level qualifies,
// Lv is left as it is.  PIMUL_EINVAL if a pair outgrew its planned transform
// (the caller then takes the host-staged path).
// PIMUL_PI_MERGED_LEVELS=0 runs those levels through pimul_sum_batch instead;
// PIMUL_PI_LEVEL_GRAPH=0 launches the merged levels one by one on the stream
// instead of through the captured graph (same kernels, for profilers that
// do not follow graph capture on several host threads).
static bool merged_levels_on() {
  const char* e = getenv("PIMUL_PI_MERGED_LEVELS");
  return !e || atoi(e) != 0;
}
static bool level_graph_on() {
  const char* e = getenv("PIMUL_PI_LEVEL_GRAPH");
  return !e || atoi(e) != 0;
}

static int merge_low_levels(DLevel& Lv, uint32_t sp, uint32_t sq, uint32_t st, size_t stop, cudaStream_t sw) {
  std::vector<DNode>& nodes = Lv.nodes;
  const size_t n0 = nodes.size();
  if (n0 < 2 || n0 > 0xFFFFFFFFull) return PIMUL_OK;
  for (size_t i = 0; i + 1 < n0; i++)
    if (nodes[i].terms & 1) return PIMUL_OK;
  // plan: per-node upper bounds of the lengths, level by level
  struct B3 {
    uint64_t p, q, t;
  };
  std::vector<B3> bnd(n0);
  for (size_t i = 0; i < n0; i++) bnd[i] = B3{nodes[i].pn, nodes[i].qn, nodes[i].tn};
  struct Plan {
    uint32_t n_in, op, oq, ot;
    int L;
  };
  std::vector<Plan> plan;
  uint64_t cp = sp, cq = sq, ct = st;
  size_t n = n0;
  while (n > std::max<size_t>(stop, 1) && n >= 2) {
    const size_t np = n / 2;
    std::vector<B3> nb(np + (n & 1));
    uint64_t need = 0;
    for (size_t i = 0; i < np; i++) {
      const B3& l = bnd[2 * i];
      const B3& r = bnd[2 * i + 1];
      const uint64_t tm = std::max(l.t + r.q, l.p + r.t);
      nb[i] = B3{l.p + r.p, l.q + r.q, tm + 1};
      need = std::max(need, 4 * std::max(std::max(l.p + r.p, l.q + r.q), tm) - 1);
    }
    if (n & 1) nb[np] = bnd[n - 1];
    int L = pimerge::MIN_LOG;
    while ((1ull << L) < need) L++;
    if (L > pimerge::MAX_LOG) break;
    uint64_t op = cp, oq = cq, ot = ct;
    for (const B3& z : nb) op = std::max(op, z.p), oq = std::max(oq, z.q), ot = std::max(ot, z.t);
    plan.push_back(Plan{(uint32_t)n, (uint32_t)op, (uint32_t)oq, (uint32_t)ot, L});
    cp = op, cq = oq, ct = ot;
    bnd.swap(nb);
    n = bnd.size();
  }
  if (plan.empty()) return PIMUL_OK;
  const double t0 = now_ms();
  int rc = PIMUL_OK;
  auto cu = [&](cudaError_t e) {
    if (e != cudaSuccess && !rc) rc = PIMUL_ECUDA;
    return e == cudaSuccess;
  };
  // device lengths of the leaves, and per merged level its slots and lengths
  const size_t K = plan.size();
  std::vector<uint64_t*> arena(K + 1, nullptr);
  std::vector<uint32_t*> lens(K + 1, nullptr);
  arena[0] = nodes[0].p;
  int* d_bad = nullptr;
  std::vector<uint32_t> h0(3 * n0);
  for (size_t i = 0; i < n0; i++) {
    h0[3 * i] = (uint32_t)nodes[i].pn;
    h0[3 * i + 1] = (uint32_t)nodes[i].qn;
    h0[3 * i + 2] = (uint32_t)nodes[i].tn;
  }
  cu(cudaMallocAsync((void**)&d_bad, 256, sw));
  cu(cudaMallocAsync((void**)&lens[0], 3 * n0 * 4, sw));
  if (!rc) cu(cudaMemcpyAsync(lens[0], h0.data(), 3 * n0 * 4, cudaMemcpyHostToDevice, sw));
  for (size_t j = 0; j < K && !rc; j++) {
    const Plan& P = plan[j];
    const size_t nn = P.n_in / 2 + (P.n_in & 1);
    if (!cu(cudaMallocAsync((void**)&arena[j + 1], nn * ((size_t)P.op + P.oq + P.ot) * 8, sw))) break;
    cu(cudaMallocAsync((void**)&lens[j + 1], 3 * nn * 4, sw));
  }
  // the schedule: every merged level back to back, captured once as a graph
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  if (!rc) rc = pimerge::prepare();
  auto enqueue = [&]() -> int {
    int crc = cudaMemsetAsync(d_bad, 0, sizeof(int), sw) == cudaSuccess ? PIMUL_OK : PIMUL_ECUDA;
    uint32_t s_p = sp, s_q = sq, s_t = st;
    for (size_t j = 0; j < K && !crc; j++) {
      const Plan& P = plan[j];
      pimerge::Level lv{arena[j], lens[j], arena[j + 1], lens[j + 1], s_p, s_q, s_t, P.op, P.oq, P.ot, P.n_in, P.L};
      crc = pimerge::merge_level(lv, d_bad, sw);
      s_p = P.op, s_q = P.oq, s_t = P.ot;
    }
    return crc;
  };
  if (!rc && !level_graph_on()) {
    rc = enqueue();
  } else if (!rc && cu(cudaStreamBeginCapture(sw, cudaStreamCaptureModeThreadLocal))) {
    const int crc = enqueue();
    const bool ended = cu(cudaStreamEndCapture(sw, &graph));
    if (!rc && crc) rc = crc;
    if (!rc && ended) cu(cudaGraphInstantiate(&exec, graph, 0));
    if (!rc) cu(cudaGraphLaunch(exec, sw));
  }
  // the last merged level's lengths and the error flag come back once
  const size_t nK = bnd.size();
  std::vector<uint32_t> hK(3 * nK);
  int h_bad = 0;
  if (!rc) cu(cudaMemcpyAsync(hK.data(), lens[K], 3 * nK * 4, cudaMemcpyDeviceToHost, sw));
  if (!rc) cu(cudaMemcpyAsync(&h_bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, sw));
  cu(cudaStreamSynchronize(sw));
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  for (size_t j = 0; j <= K; j++)
    if (lens[j]) cudaFreeAsync(lens[j], sw);
  if (d_bad) cudaFreeAsync(d_bad, sw);
  for (size_t j = 1; j < K; j++)
    if (arena[j]) cudaFreeAsync(arena[j], sw);
  if (!rc && h_bad) rc = PIMUL_EINVAL;
  if (rc) {
    if (arena[K]) cudaFreeAsync(arena[K], sw);
    return rc;
  }
  // the new level: slots of the last plan, terms summed pairwise
  std::vector<uint64_t> terms(n0);
  for (size_t i = 0; i < n0; i++) terms[i] = nodes[i].terms;
  for (size_t j = 0; j < K; j++) {
    std::vector<uint64_t> nt(terms.size() / 2 + (terms.size() & 1));
    for (size_t i = 0; i + 1 < terms.size(); i += 2) nt[i / 2] = terms[i] + terms[i + 1];
    if (terms.size() & 1) nt.back() = terms.back();
    terms.swap(nt);
  }
  const Plan& PK = plan.back();
  const size_t stride = (size_t)PK.op + PK.oq + PK.ot;
  std::vector<DNode> next(nK);
  for (size_t i = 0; i < nK; i++) {
    DNode& z = next[i];
    z.p = arena[K] + i * stride;
    z.q = z.p + PK.op;
    z.t = z.q + PK.oq;
    z.pn = hK[3 * i], z.qn = hK[3 * i + 1], z.tn = hK[3 * i + 2];
    z.terms = terms[i];
  }
  for (uint64_t* a : Lv.arenas) cudaFreeAsync(a, sw);
  Lv.arenas.assign(1, arena[K]);
  nodes.swap(next);
  uint64_t npairs = 0;
  for (size_t j = 0; j < K; j++) {
    const uint64_t pairs = plan[j].n_in / 2;
    npairs += pairs;
    C().ntt_hist[plan[j].L].fetch_add(4 * pairs, std::memory_order_relaxed);
  }
  C().ntt_calls.fetch_add(4 * npairs, std::memory_order_relaxed);
  C().batch_levels.fetch_add(K, std::memory_order_relaxed);
  const double t1 = now_ms();
  bt_add(1, t1 - t0);
  if (getenv("PIMUL_PI_TIMING"))
    fprintf(stderr, "[pimul]   merged levels: %zu (from %zu nodes to %zu, transforms 2^%d..2^%d), %.1f ms\n", K, n0,
            nK, plan.front().L, plan.back().L, t1 - t0);
  return PIMUL_OK;
}

// Device-resident splitting over terms [a, b): segment by segment, the
// leaves are computed on the device (leaves.cu) into fixed slots and the
// segment is reduced to its root; the segment roots are then merged on the
// device and only the final Q and |T| come back, or, with keep, stay on the
// device (keep->lvl.nodes[0], arenas owned by keep).  Returns PIMUL_EINVAL
// (the caller then takes the host-staged path) if a leaf breaks the static
// signs or outgrows its slot, or a leaf is longer than the kernel takes.
static int split_root_device(uint64_t a, uint64_t b, uint64_t leaf, Int& q, Int& t, DevRoot* keep) {
  // eight equal term ranges, each with its own leaf size: the GPU starts
  // after an eighth of the leaves (Q and T of a range do not depend on
  // where it is split, so neither do the results)
  const size_t nseg = (b - a) / 32 >= 128 ? 8 : 1;
  std::vector<uint64_t> seg_k(nseg + 1), seg_leaf(nseg);
  // even term counts before every boundary, so that merged left nodes have
  // an even number of terms and their T is a sum (fused on the device)
  for (size_t s = 0; s < nseg; s++) seg_k[s] = a + (((b - a) * s / nseg) & ~1ull);
  seg_k[nseg] = b;
  for (size_t s = 0; s < nseg; s++) seg_leaf[s] = leaf == LEAF_AUTO ? 2 * auto_leaf(seg_k[s + 1]) : leaf;
  // the splitting's stream has the highest priority: the products of the
  // threads running beside it (sqrt(10005), the decimal scale, the
  // conversion's divisors) fill the gaps between its levels instead of
  // slowing them down
  int prio_lo = 0, prio_hi = 0;
  cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi);
  cudaStream_t st = nullptr;
  if (cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, prio_hi) != cudaSuccess) return PIMUL_ECUDA;
  std::vector<DLevel> roots(nseg);
  std::vector<double> seg_tl(nseg, 0.0);
  // one segment: leaves on the device, then its levels (stopping at `stop`
  // nodes), all on stream sw
  auto run_segment = [&](size_t sgi, cudaStream_t sw) -> int {
    const uint64_t k0 = seg_k[sgi], k1 = seg_k[sgi + 1], lf = seg_leaf[sgi];
    if (lf > pileaf::MAX_TERMS) return PIMUL_EINVAL;
    const uint64_t nl = (k1 - k0 + lf - 1) / lf;
    double t0 = now_ms();
    // slots sized from the segment's last full leaf (the largest values),
    // plus two limbs; a leaf that outgrows its slot is reported, not written
    const uint64_t kl = k1 - k0 >= lf ? k0 + ((k1 - k0) / lf - 1) * lf : k0;
    const PQT big = split_leaf(kl, std::min(k1, kl + lf));
    const uint32_t sp = (uint32_t)big.p.m.size() + 2, sq = (uint32_t)big.q.m.size() + 2,
                   stt = (uint32_t)big.t.m.size() + 2;
    uint64_t* arena = nullptr;
    if (cudaMallocAsync((void**)&arena, std::max<uint64_t>(nl * (sp + sq + stt), 1) * 8, sw) != cudaSuccess) {
      cudaGetLastError();
      return PIMUL_ENOMEM;
    }
    roots[sgi].arenas.push_back(arena);
    std::vector<uint32_t> lens(3 * nl);
    std::vector<uint8_t> signs(nl);
    int rc = pileaf::leaves_device(k0, k1, (uint32_t)lf, (uint32_t)nl, sp, sq, stt, arena, lens.data(), signs.data(), sw);
    seg_tl[sgi] = now_ms() - t0;
    if (rc) return rc;
    std::vector<DNode>& nodes = roots[sgi].nodes;
    nodes.resize(nl);
    for (uint64_t i = 0; i < nl && !rc; i++) {
      const uint64_t terms = std::min(k1, k0 + (i + 1) * lf) - (k0 + i * lf);
      // static signs: T < 0 and P of m terms has sign (-1)^m
      if (!(signs[i] & 2) || (bool)(signs[i] & 1) != (bool)(terms & 1)) rc = PIMUL_EINVAL;
      DNode& nd = nodes[i];
      nd.p = arena + i * (sp + sq + stt);
      nd.q = nd.p + sp;
      nd.t = nd.q + sq;
      nd.pn = lens[3 * i], nd.qn = lens[3 * i + 1], nd.tn = lens[3 * i + 2];
      nd.terms = terms;
    }
    // served mode: each segment stops at its share of the nodes handed to the service
    const size_t stop = C().serve_nodes && keep ? std::max<size_t>(1, C().serve_nodes / nseg) : 1;
    if (!rc && merged_levels_on()) rc = merge_low_levels(roots[sgi], sp, sq, stt, stop, sw);
    if (!rc) rc = dev_reduce(roots[sgi], sw, true, stop);
    return rc;
  };
  // segments on two host threads with a stream each: one segment's host work
  // (leaf slots, descriptors, the level lengths read back) overlaps the
  // other's kernels
  const size_t nwork = nseg >= 2 ? 2 : 1;
  std::vector<cudaStream_t> wst(nwork, st);
  for (size_t w = 1; w < nwork; w++)
    if (cudaStreamCreateWithPriority(&wst[w], cudaStreamNonBlocking, prio_hi) != cudaSuccess) wst[w] = nullptr;
  std::atomic<size_t> next_seg{0};
  std::atomic<int> seg_rc{0};
  auto work = [&](size_t w) {
    for (;;) {
      const size_t sgi = next_seg.fetch_add(1);
      if (sgi >= nseg || seg_rc.load()) break;
      const int r = wst[w] ? run_segment(sgi, wst[w]) : PIMUL_ECUDA;
      int none = 0;
      if (r) seg_rc.compare_exchange_strong(none, r);
    }
  };
  {
    std::list<Worker> helpers;
    for (size_t w = 1; w < nwork; w++) helpers.emplace_back([&work, w] { work(w); });
    work(0);
    for (Worker& h : helpers) h.join();
  }
  for (size_t w = 1; w < nwork; w++)
    if (wst[w]) {
      cudaStreamSynchronize(wst[w]);
      cudaStreamDestroy(wst[w]);
    }
  int rc = seg_rc.load();
  double tl = 0;
  for (double x : seg_tl) tl += x;
  C().leaf_ms += tl;
  DLevel top;
  for (DLevel& r : roots) {
    for (const DNode& n : r.nodes) top.nodes.push_back(n);
    top.arenas.insert(top.arenas.end(), r.arenas.begin(), r.arenas.end());
  }
  if (keep && C().serve_nodes && !rc) {
    rc = serve_root(top, st, keep);
    cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
    keep->lvl.arenas = std::move(top.arenas);  // the handed-over nodes: freed after the final assembly
    return rc;
  }
  if (keep && keep->top_limbs && !rc) {
    rc = dev_reduce(top, st, true, 2);
    if (!rc && top.nodes.size() == 2) rc = dev_root_truncated(top, st, keep->top_limbs, keep);
  }
  if (!rc) rc = dev_reduce(top, st, false);
  if (!rc && keep) {
    cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
    keep->lvl = std::move(top);
    return PIMUL_OK;
  }
  if (!rc) {
    double t0 = now_ms();
    const DNode& r = top.nodes[0];
    Limbs qm(r.qn), tm(r.tn);
    if (cudaMemcpyAsync(qm.data(), r.q, r.qn * 8, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaMemcpyAsync(tm.data(), r.t, r.tn * 8, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      rc = PIMUL_ECUDA;
    q = Int(std::move(qm), false);
    t = Int(std::move(tm), true);
    bt_add(2, now_ms() - t0);
  }
  dev_free(top, st);
  cudaStreamSynchronize(st);
  cudaStreamDestroy(st);
  return rc;
}

static int split_root_batched(uint64_t a, uint64_t b, uint64_t leaf, Int& q, Int& t, DevRoot* keep = nullptr) {
  const uint64_t nleaf = (b - a + (leaf == LEAF_AUTO ? 32 : leaf) - 1) / (leaf == LEAF_AUTO ? 32 : leaf);
  for (double& x : C().bt) x = 0;
  C().leaf_ms = 0;
  // device-resident levels (every range obeys the static signs; a leaf that
  // did not would send the splitting down the host-staged path below)
  if (nleaf > 1) {
    int rc = split_root_device(a, b, leaf, q, t, keep);
    report_split("binary splitting (device-resident levels)");
    if (rc != PIMUL_EINVAL) return rc;
  }
  if (leaf == LEAF_AUTO) leaf = 32;
  std::vector<PQT> nodes(nleaf);
  double t0 = now_ms();
  parallel_for(nleaf, [&](size_t lo, size_t hi) {
    for (size_t i = lo; i < hi; i++) nodes[i] = split(a + i * leaf, std::min(b, a + (i + 1) * leaf), 4);
  });
  C().leaf_ms = now_ms() - t0;
  LevelStaging S;
  int rc = S.init();
  while (!rc && nodes.size() > 1) rc = merge_level(nodes, S);
  if (rc) return rc;
  q = std::move(nodes[0].q);
  t = std::move(nodes[0].t);
  report_split("binary splitting");
  return PIMUL_OK;
}

// ------------------------------------------------ batched decimal conversion
// Level-synchronous divide and conquer on C = 10^19: with P_k = C^(2^k),
// every node of level k (a value below P_k^2) splits into (q, r) = divmod by
// P_k, high half first.  All nodes of a level share P_k and one reciprocal
// V_k <= 2^s / P_k (s = 2 bits(P_k) + 64), so floor(N V_k / 2^s) is the
// quotient or one less.  The levels run on the device with the nodes in HBM
// (dec.cu): the value goes up once and only the digits come back.  An
// integer has one decimal string, so the output equals the reference's
// conversion (crates/bignum/src/integer.rs:892-983).
// The divisors and reciprocals of the levels depend only on the number of
// chunks, so a caller that knows the digit count can build them early.
struct DecPlan {
  int K = 0, kmin = 0;
  std::vector<Int> P;       // P_k = (10^19)^(2^k)
  std::vector<Int> V;       // V_k ~ 2^(s_k) / P_k, k >= kmin
  std::vector<uint64_t> sh; // s_k = 2 bits(P_k) + 64
  pidec::DevLevels dev;     // or: levels kmin..K-1 built in device memory (dev.K == K)
};

// Plan for integers of at most ndig decimal digits.  V_k: Newton once at the
// top, corrected to exactly floor(2^s / P), then V_(k-1) = (P_(k-1) V_k) >>
// (s_k - s_(k-1)), which stays at or below floor(2^(s_(k-1)) / P_(k-1))
// since P_k = P_(k-1)^2 and is within two units of it.  So every quotient
// estimate floor(x V_k / 2^(s_k)) is at most x div P_k and, for x < P_k^2,
// short of it by less than 2^-63 before the floor.
static DecPlan make_dec_plan(uint64_t ndig) {
  DecPlan D;
  const uint64_t nch = (ndig + 18) / 19;
  while ((1ull << D.K) < nch) D.K++;
  D.kmin = std::min(D.K, pidec::LEAF_K);
  D.P.resize(D.K);
  D.V.resize(D.K);
  D.sh.resize(D.K);
  if (D.K == 0) return D;
  D.P[0] = Int(DEC_CHUNK);
  for (int k = 1; k < D.K; k++) D.P[k] = mul(D.P[k - 1], D.P[k - 1]);
  for (int k = D.K - 1; k >= D.kmin; k--) {
    const uint64_t b = bits_of(D.P[k].m);
    D.sh[k] = 2 * b + 64;
    if (k == D.K - 1) {
      Flt r = reciprocal_at_prec(flt_from_int(D.P[k]), b + 128);
      r.exp += (int64_t)D.sh[k];
      D.V[k] = to_integer_down(r);
      // P V <= 2^s < P (V + 1)
      const Limbs two_s = shl_mag(Limbs(1, 1), D.sh[k]);
      Limbs pv = mul_mag(D.P[k].m, D.V[k].m);
      while (cmp_mag(pv, two_s) > 0) {
        D.V[k] = sub(D.V[k], Int(1));
        pv = sub_mag(pv, D.P[k].m);
      }
      for (;;) {
        Limbs up = add_mag(pv, D.P[k].m);
        if (cmp_mag(up, two_s) > 0) break;
        D.V[k] = add(D.V[k], Int(1));
        pv = std::move(up);
      }
    } else {
      D.V[k] = Int(shr_mag(mul_mag(D.P[k].m, D.V[k + 1].m), D.sh[k + 1] - D.sh[k]), false);
    }
  }
  return D;
}

// The same plan with its levels built on the device (pidec::build_levels_device:
// every V_k an underestimate within a few units of floor(2^(s_k) / P_k),
// which the conversion's correction rounds absorb); a small plan is built on
// the host.
static DecPlan make_dec_plan_device(uint64_t ndig) {
  DecPlan D;
  const uint64_t nch = (ndig + 18) / 19;
  while ((1ull << D.K) < nch) D.K++;
  if (D.K <= pidec::LEAF_K) return make_dec_plan(ndig);
  D.kmin = pidec::LEAF_K;
  const int rc = pidec::build_levels_device(D.K, &D.dev, nullptr);
  if (rc) {
    int none = 0;
    C().error.compare_exchange_strong(none, rc);
    throw PiAbort{rc};
  }
  return D;
}

// Exactly `want` decimal digits of x < 10^want (zero-padded on the left),
// written straight into out; x: n limbs on the host, or in device memory
// (on_dev), of bit length xbits.
static int to_decimal_core(const uint64_t* x, size_t n, bool on_dev, uint64_t xbits, char* out, size_t want,
                           const DecPlan* plan) {
  DecPlan own;
  const uint64_t ndig = std::max<uint64_t>(dec_estimate(xbits) + 1, want);
  if (!plan || (1ull << plan->K) * 19 < ndig) {
    own = make_dec_plan(ndig);
    plan = &own;
  }
  if (C().error.load()) return C().error.load();
  if (plan->kmin != pidec::LEAF_K) return PIMUL_EINVAL;
  const size_t total = (size_t)19 << plan->K;
  if (want > total) {
    memset(out, '0', want - total);
    out += want - total;
    want = total;
  }
  const bool lv_dev = plan->dev.K == plan->K;
  std::vector<pidec::Level> lv(plan->K);
  if (!lv_dev)
    for (int k = plan->kmin; k < plan->K; k++)
      lv[k] = pidec::Level{plan->P[k].m.data(), plan->P[k].m.size(), plan->V[k].m.data(), plan->V[k].m.size(),
                           plan->sh[k]};
  double ms[3] = {0, 0, 0};
  int rc = pidec::to_decimal_device(x, n, on_dev, plan->K, lv_dev ? plan->dev.lv.data() : lv.data(), lv_dev, out,
                                    want, ms);
  if (getenv("PIMUL_PI_TIMING"))
    fprintf(stderr, "[pimul] decimal conversion on the device: upload %.1f ms, levels %.1f, leaves + download %.1f\n",
            ms[0], ms[1], ms[2]);
  return rc;
}

// Exactly `want` decimal digits of X < 10^want (zero-padded on the left),
// written straight into out.
static int to_decimal_batched_into(const Int& X, char* out, size_t want, const DecPlan* plan) {
  if (X.m.size() <= 256) {
    std::string s = to_decimal_top(X);
    if (s.size() > want) return PIMUL_EINVAL;
    memset(out, '0', want - s.size());
    memcpy(out + want - s.size(), s.data(), s.size());
    return C().error.load();
  }
  return to_decimal_core(X.m.data(), X.m.size(), false, bits_of(X.m), out, want, plan);
}

// The same for a trimmed integer of n limbs in device memory.
static int to_decimal_batched_into_dev(const uint64_t* dx, size_t n, char* out, size_t want, const DecPlan* plan) {
  if (n <= 256) {
    Limbs h(n);
    if (n && cudaMemcpy(h.data(), dx, n * 8, cudaMemcpyDeviceToHost) != cudaSuccess) return PIMUL_ECUDA;
    return to_decimal_batched_into(Int(std::move(h), false), out, want, plan);
  }
  uint64_t top = 0;
  if (cudaMemcpy(&top, dx + (n - 1), 8, cudaMemcpyDeviceToHost) != cudaSuccess) return PIMUL_ECUDA;
  const uint64_t xbits = 64 * (uint64_t)(n - 1) + (top ? 64 - __builtin_clzll(top) : 0);
  return to_decimal_core(dx, n, true, xbits, out, want, plan);
}

static int to_decimal_batched(const Int& X, std::string& outs) {
  std::string all(dec_estimate(bits_of(X.m)) + 1, '0');
  int rc = to_decimal_batched_into(X, &all[0], all.size(), nullptr);
  if (rc) return rc;
  size_t nz = all.find_first_not_of('0');
  outs = nz == std::string::npos ? std::string("0") : all.substr(nz);
  return PIMUL_OK;
}

}  // namespace pihost

using namespace pihost;

static int finish_digits(Flt pi, const Flt& scale, uint64_t digits, char* out, double* t_phase,
                         const DecPlan* device_plan = nullptr) {
  double t0 = now_ms();
  pi = mul_at_prec(pi, scale, pi.prec);
  Int ip = to_integer_down(pi);
  if (device_plan) {
    int rc = to_decimal_batched_into(ip, out, digits, device_plan);
    if (t_phase) *t_phase = now_ms() - t0;
    return rc ? rc : C().error.load();
  }
  std::string s = to_decimal_top(ip);
  if (t_phase) *t_phase = now_ms() - t0;
  if (C().error.load()) return C().error.load();
  if (s.size() < digits) s = std::string(digits - s.size(), '0') + s;
  memcpy(out, s.data(), digits);
  return PIMUL_OK;
}

// Digits of pi by Gauss-Legendre (see pimul.h).
static int gauss_legendre_body(uint64_t digits, char* out, uint32_t flags, double* phase_ms,
                               uint64_t* ntt_products) {
  const uint64_t prec = (uint64_t)std::ceil((double)digits * 3.321928094887362) + 256;
  double t0 = now_ms();
  if (flags & PIMUL_PI_DEVICE_AGM) {
    // the AGM, the quotient and the conversion on the device; the decimal
    // scale 10^(D-1) = 5^(D-1) 2^(D-1) (5^(D-1) exact, on the device) and the
    // conversion's divisors on threads beside the iteration
    piagm::DevNum p5;
    int p5rc = PIMUL_OK;
    Worker scale_th([&] { p5rc = piagm::pow5_device(digits - 1, &p5); });
    DecPlan dplan;
    Worker plan_th([&] { dplan = make_dec_plan_device(digits + 1); });
    piagm::AgmOut A;
    int rc = piagm::agm_device(prec, &A, nullptr);
    const double t1 = now_ms();
    scale_th.join();
    plan_th.join();
    uint64_t* d_ip = nullptr;
    size_t ipn = 0;
    if (!rc) rc = p5rc;
    if (!rc && C().error.load()) rc = C().error.load();
    if (!rc) {
      // pi 10^(D-1) = 5^(D-1) 2^(D-3) (a + b)^2 / t
      const size_t nl = (prec + 192 + 63) / 64, lq = std::min(A.num_limbs, nl);
      rc = pidec::quotient_device(A.den, A.den_limbs, A.den_exp, A.num + (A.num_limbs - lq), lq,
                                  A.num_exp + 64 * (int64_t)(A.num_limbs - lq), p5.mant, p5.limbs,
                                  (int64_t)digits - 3, true, prec, &d_ip, &ipn, nullptr);
    }
    if (p5.mant) cudaFree(p5.mant);
    if (A.num) cudaFree(A.num);
    if (A.den) cudaFree(A.den);
    if (!rc) rc = to_decimal_batched_into_dev(d_ip, ipn, out, digits, &dplan);
    if (d_ip) cudaFree(d_ip);
    if (phase_ms) {
      phase_ms[0] = t1 - t0;
      phase_ms[1] = 0;
      phase_ms[2] = now_ms() - t1;
    }
    if (ntt_products) *ntt_products = C().ntt_calls.load();
    return rc;
  }
  // the decimal scale 10^(D-1) at the working precision runs beside the
  // iterations (it depends on nothing else)
  Flt scale;
  Worker scale_th([&] { scale = pow_int(flt_from_u64(10, prec), Int(digits - 1)); });
  // the device conversion's divisors and reciprocals too
  const bool device_dec = (flags & PIMUL_PI_DEVICE_DECIMAL) != 0;
  DecPlan dplan;
  Worker plan_th([&] {
    if (device_dec) dplan = make_dec_plan(digits + 1);
  });
  Flt pi = gauss_legendre(prec, (flags & PIMUL_PI_FAST_SQRT) != 0);
  double t1 = now_ms();
  scale_th.join();
  plan_th.join();
  double tdc = 0;
  int rc = finish_digits(pi, scale, digits, out, &tdc, device_dec ? &dplan : nullptr);
  if (phase_ms) {
    phase_ms[0] = t1 - t0;
    phase_ms[1] = 0;
    phase_ms[2] = tdc;
  }
  if (ntt_products) *ntt_products = C().ntt_calls.load();
  return rc;
}

extern "C" int pimul_pi_gauss_legendre_ex(uint64_t digits, char* out, size_t cap, pimul_mul_fn backend,
                                          uint64_t ntt_threshold, uint32_t flags, double* phase_ms,
                                          uint64_t* ntt_products) {
  if (digits == 0) return PIMUL_OK;
  if (!out || cap < digits) return PIMUL_EINVAL;
  PiCtx ctx;
  ctx.backend = reinterpret_cast<mul_fn>(backend);
  ctx.ntt_threshold = ntt_threshold ? ntt_threshold : 8192;
  return with_ctx(ctx, [&] { return gauss_legendre_body(digits, out, flags, phase_ms, ntt_products); });
}

extern "C" int pimul_pi_gauss_legendre(uint64_t digits, char* out, size_t cap, pimul_mul_fn backend,
                                       uint64_t ntt_threshold, double* phase_ms, uint64_t* ntt_products) {
  return pimul_pi_gauss_legendre_ex(digits, out, cap, backend, ntt_threshold, 0, phase_ms, ntt_products);
}

// Digits of pi by Chudnovsky (crates/pi-core/src/algorithm/chudnovsky.rs:75-235):
// writes `digits` characters ("31415...", no decimal point) to out.
// phase_ms (optional, 3 entries): binary splitting, final assembly,
// decimal conversion.  backend NULL = the GPU engine (pimul_mul).
static int chudnovsky_body(uint64_t digits, char* out, uint64_t leaf_terms, double* phase_ms,
                           uint64_t* ntt_products, uint64_t* ntt_hist33) {
  // precision.rs:64: bits = ceil(D log2 10) + 256
  const uint64_t prec = (uint64_t)std::ceil((double)digits * 3.321928094887362) + 256;
  const uint64_t n_terms = (uint64_t)std::ceil((double)digits / DIGITS_PER_TERM) + SAFETY_TERMS;
  double t0 = now_ms();
  // sqrt(10005) * 426880 runs beside the binary splitting (chudnovsky.rs:118-126),
  // and so does the decimal scale 10^(D-1) at the working precision, which
  // depends on nothing else (util.rs:25-83 computes it after pi).  The plain
  // form computes both on the host (sqrt_mut restates the reference's
  // iteration); the batched form computes their product
  // W = 426880 sqrt(10005) 10^(D-1) on the device for the device final
  // assembly, and both host values only if the splitting ends on the host.
  Flt sq, scale;
  double t_sqrt = 0, t_scale = 0, t_w = 0, t_plan = 0;
  auto host_sqrt = [&] {
    double ts = now_ms();
    Flt p;
    if (leaf_terms) {
      p = sqrt_int_fast(10005, prec);
    } else {
      p = flt_from_u64(10005, prec);
      sqrt_mut(p);
    }
    sq = mul_at_prec(p, flt_from_u64(426880, 64), p.prec);
    t_sqrt = now_ms() - ts;
  };
  auto host_scale = [&] {
    double ts = now_ms();
    scale = pow_int(flt_from_u64(10, prec), Int(digits - 1));
    t_scale = now_ms() - ts;
  };
  Worker sqrt_th, scale_th;
  if (!leaf_terms) {
    sqrt_th.start(host_sqrt);
    scale_th.start(host_scale);
  }
  // batched form: the decimal conversion's divisors and reciprocals too
  DecPlan dplan;
  Worker plan_th([&] {
    double ts = now_ms();
    if (leaf_terms) dplan = make_dec_plan_device(digits + 1);
    t_plan = now_ms() - ts;
  });
  piagm::DevNum W;
  int w_rc = PIMUL_OK;
  Worker w_th;
  if (leaf_terms)
    w_th.start([&] {
      double ts = now_ms();
      w_rc = piagm::chudnovsky_w_device(digits, prec, &W, nullptr);
      t_w = now_ms() - ts;
    });
  struct WGuard {  // the device W, whichever way this call ends
    Worker& th;
    piagm::DevNum& w;
    ~WGuard() {
      try {
        th.join();
      } catch (...) {
      }
      if (w.mant) cudaFree(w.mant);
      w.mant = nullptr;
    }
  } w_guard{w_th, W};
  // the host values, for the plain form or a batched splitting that ended on the host
  auto join_sqrt = [&] {
    if (!leaf_terms) {
      sqrt_th.join();
    } else if (sq.zero()) {
      Worker sc(host_scale);
      host_sqrt();
      sc.join();
    }
  };
  auto join_scale = [&] {
    if (!leaf_terms) scale_th.join();
  };
  Int q, t;
  DevRoot droot;  // the root's Q and |T| when they stay on the device
  struct ArenaGuard {  // returns the root's arenas and service handles when an error ends this call
    DevRoot& R;
    ~ArenaGuard() {
      for (uint64_t h : R.svc_handles) pimul_free(h);
      R.svc_handles.clear();
      for (uint64_t* ar : R.lvl.arenas) cudaFree(ar);
      R.lvl.arenas.clear();
    }
  } arena_guard{droot};
  droot.top_limbs = pidec::final_assembly_top_limbs(prec);
  int brc = PIMUL_OK;
  if (leaf_terms)
    brc = split_root_batched(1, n_terms + 1, leaf_terms, q, t, &droot);
  else
    split_root(1, n_terms + 1, q, t);
  if (brc) {
    for (uint64_t* ar : droot.lvl.arenas) cudaFree(ar);
    droot.lvl.arenas.clear();
    if (!leaf_terms) {
      sqrt_th.join();
      scale_th.join();
    }
    plan_th.join();
    return brc;
  }
  double t1 = now_ms();
  if (!droot.lvl.nodes.empty()) {
    // final assembly and decimal conversion without leaving the device
    w_th.join();
    const DNode& r = droot.lvl.nodes[0];
    uint64_t* d_ip = nullptr;
    size_t ipn = 0;
    double fms[2] = {0, 0};
    int frc = w_rc;
    if (!frc)
      frc = pidec::final_assembly_device(r.q, r.qn, droot.q_off, r.t, r.tn, droot.t_off, CH_A, W.mant, W.limbs, W.exp,
                                         true, prec, &d_ip, &ipn, fms);
    for (uint64_t h : droot.svc_handles) pimul_free(h);
    droot.svc_handles.clear();
    for (uint64_t* ar : droot.lvl.arenas) cudaFree(ar);
    droot.lvl.arenas.clear();
    double t2 = now_ms();
    plan_th.join();
    if (!frc) frc = to_decimal_batched_into_dev(d_ip, ipn, out, digits, &dplan);
    if (d_ip) cudaFree(d_ip);
    double t3 = now_ms();
    if (getenv("PIMUL_PI_TIMING"))
      fprintf(stderr, "[pimul] W thread %.1f ms, conversion plan thread %.1f ms, final assembly on the device: "
              "reciprocal %.1f ms, products %.1f ms\n", t_w, t_plan, fms[0], fms[1]);
    if (frc) return frc;
    if (C().error.load()) return C().error.load();
    if (phase_ms) {
      phase_ms[0] = t1 - t0;
      phase_ms[1] = t2 - t1;
      phase_ms[2] = t3 - t2;
    }
    if (ntt_products) *ntt_products = C().ntt_calls.load();
    if (ntt_hist33)
      for (int i = 0; i < 33; i++) ntt_hist33[i] = C().ntt_hist[i].load();
    return PIMUL_OK;
  }
  // final assembly (chudnovsky.rs:146-204)
  Int denom = add(mul(Int(CH_A), q), t);
  Flt denf = flt_from_int(denom);
  Flt recip = reciprocal_at_prec(denf, prec + 16);
  double t_recip = now_ms() - t1;
  join_sqrt();
  Flt num = mul_at_prec(sq, flt_from_int(q), sq.prec);
  Flt pi = mul_at_prec(num, recip, prec);
  double t2 = now_ms();
  // decimal conversion (util.rs:25-83)
  join_scale();
  double t_join = now_ms() - t2;
  pi = mul_at_prec(pi, scale, pi.prec);
  Int ip = to_integer_down(pi);
  std::string s;
  plan_th.join();
  bool written = false;
  if (leaf_terms) {
    int crc = to_decimal_batched_into(ip, out, digits, &dplan);
    if (crc) return crc;
    written = true;
  } else {
    s = to_decimal_top(ip);
  }
  double t3 = now_ms();
  if (getenv("PIMUL_PI_TIMING"))
    fprintf(stderr, "[pimul] sqrt thread %.1f ms, scale thread %.1f ms (waited %.1f), reciprocal %.1f ms\n", t_sqrt,
            t_scale, t_join, t_recip);
  if (C().error.load()) return C().error.load();
  if (!written) {
    if (s.size() < digits) s = std::string(digits - s.size(), '0') + s;
    memcpy(out, s.data(), digits);
  }
  if (phase_ms) {
    phase_ms[0] = t1 - t0;
    phase_ms[1] = t2 - t1;
    phase_ms[2] = t3 - t2;
  }
  if (ntt_products) *ntt_products = C().ntt_calls.load();
  if (ntt_hist33)
    for (int i = 0; i < 33; i++) ntt_hist33[i] = C().ntt_hist[i].load();
  return PIMUL_OK;
}

static int chudnovsky(uint64_t digits, char* out, size_t cap, pimul_mul_fn backend, uint64_t ntt_threshold,
                      uint64_t leaf_terms, double* phase_ms, uint64_t* ntt_products, uint64_t* ntt_hist33,
                      uint64_t* levels, uint64_t serve_nodes = 0, uint64_t* served_requests = nullptr) {
  if (digits == 0) return PIMUL_OK;
  if (!out || cap < digits) return PIMUL_EINVAL;
  PiCtx ctx;
  ctx.backend = reinterpret_cast<mul_fn>(backend);
  ctx.ntt_threshold = ntt_threshold ? ntt_threshold : 8192;
  ctx.serve_nodes = serve_nodes;
  const double t0 = now_ms();
  int rc = with_ctx(ctx, [&] { return chudnovsky_body(digits, out, leaf_terms, phase_ms, ntt_products, ntt_hist33); });
  if (getenv("PIMUL_PI_TIMING")) fprintf(stderr, "[pimul] driver call %.1f ms\n", now_ms() - t0);
  if (levels) *levels = ctx.batch_levels.load();
  if (served_requests) *served_requests = ctx.served_requests;
  return rc;
}

extern "C" int pimul_pi_chudnovsky(uint64_t digits, char* out, size_t cap, pimul_mul_fn backend,
                                   uint64_t ntt_threshold, double* phase_ms, uint64_t* ntt_products,
                                   uint64_t* ntt_hist33) {
  return chudnovsky(digits, out, cap, backend, ntt_threshold, 0, phase_ms, ntt_products, ntt_hist33, nullptr);
}

// Decimal string of a non-negative integer (see pimul.h).
extern "C" int pimul_to_decimal(const uint64_t* limbs, size_t n, char* out, size_t cap, size_t* len,
                                int batched) {
  if (!len || (n && !limbs)) return PIMUL_EINVAL;
  PiCtx ctx;
  return with_ctx(ctx, [&]() -> int {
    Int x(Limbs(limbs, limbs + n), false);
    std::string s;
    if (x.zero()) {
      s = "0";
    } else if (batched) {
      int rc = to_decimal_batched(x, s);
      if (rc) return rc;
    } else {
      s = to_decimal_top(x);
    }
    *len = s.size();
    if (!out || cap < s.size()) return PIMUL_EINVAL;
    memcpy(out, s.data(), s.size());
    return PIMUL_OK;
  });
}

// Batched form (see pimul.h): binary splitting level by level through
// pimul_mul_batch, everything after it as in pimul_pi_chudnovsky.
extern "C" int pimul_pi_chudnovsky_batched(uint64_t digits, char* out, size_t cap, uint64_t leaf_terms,
                                           double* phase_ms, uint64_t* gpu_products, uint64_t* levels,
                                           uint64_t* ntt_hist33) {
  return chudnovsky(digits, out, cap, nullptr, 0, leaf_terms ? leaf_terms : LEAF_AUTO, phase_ms, gpu_products,
                    ntt_hist33, levels);
}

// The splitting's upper levels through the multiply service (see pimul.h).
extern "C" int pimul_pi_chudnovsky_served(uint64_t digits, char* out, size_t cap, uint64_t serve_nodes,
                                          double* phase_ms, uint64_t* gpu_products, uint64_t* requests) {
  return chudnovsky(digits, out, cap, nullptr, 0, LEAF_AUTO, phase_ms, gpu_products, nullptr, nullptr,
                    serve_nodes ? serve_nodes : 512, requests);
}
