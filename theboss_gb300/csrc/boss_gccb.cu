// boss_gccb.cu -- batched generalized Clifford & Clifford (version B) sampling.
//
// theboss draws one sample at a time (generalized_cliffords_b_simulation_strategy.py:41-110,
// generalized_cliffords_b_uniform_losses_simulation_strategy.py:87-121): per step it pops a
// random remaining input particle, computes the all-minors permanents of the
// current input against the output so far, expands them into the m output
// probabilities and draws one output mode.  Every random number it draws depends
// only on counts, never on a probability, so the host replays numpy's MT19937
// stream first (same calls, same order; on several host threads for large
// batches) and the GPU then runs all samples level by level:
//   level k: the all-minors sweeps of every sample that has >= k particles, as
//   one launch of minors_sweep_kernel (at the last levels followed by
//   gccb_partials_reduce_kernel), then gccb_finalize_kernel (one warp per
//   sample): fixed-order reduction of the sweep partials, the Laplace expansion
//   over the m outputs (exact integer sums), |.|^2, numpy.random.choice's cdf /
//   searchsorted rule decided exactly, and the sweep plan of the sample's next
//   level.
// The whole level loop is captured into one CUDA graph and launched once; large
// calls run as pipelined parts, each with its own graph and stream.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <stdio.h>
#include <stdlib.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <functional>
#include <map>
#include <mutex>
#include <string>
#include <numeric>
#include <thread>
#include <vector>

#include "../../include/boss.h"
#include "boss_internal.h"

namespace boss {

extern std::mutex g_api_mutex;

// ---------------------------------------------------------------------------
// numpy legacy RandomState replay (MT19937, Matsumoto & Nishimura 1998).
// ---------------------------------------------------------------------------
struct MT19937 {
  uint32_t key[624];
  uint32_t out[624];  // the tempered outputs of key (the next 624 - pos draws)
  int pos;

  void temper_all() {  // one vectorisable pass per block instead of per draw
    for (int j = 0; j < 624; ++j) {
      uint32_t y = key[j];
      y ^= y >> 11;
      y ^= (y << 7) & 0x9d2c5680u;
      y ^= (y << 15) & 0xefc60000u;
      y ^= y >> 18;
      out[j] = y;
    }
  }
  void twist() {
    twist_key();
    temper_all();
    pos = 0;
  }
  void twist_key() {  // the next block's key, without tempering it
    const uint32_t upper = 0x80000000u, lower = 0x7fffffffu, a = 0x9908b0dfu;
    int i = 0;
    for (; i < 624 - 397; ++i) {
      const uint32_t y = (key[i] & upper) | (key[i + 1] & lower);
      key[i] = key[i + 397] ^ (y >> 1) ^ ((0u - (y & 1u)) & a);
    }
    for (; i < 623; ++i) {
      const uint32_t y = (key[i] & upper) | (key[i + 1] & lower);
      key[i] = key[i + 397 - 624] ^ (y >> 1) ^ ((0u - (y & 1u)) & a);
    }
    const uint32_t y = (key[623] & upper) | (key[0] & lower);
    key[623] = key[396] ^ (y >> 1) ^ ((0u - (y & 1u)) & a);
  }
  inline uint32_t next32() {
    if (pos >= 624) twist();
    return out[pos++];
  }
  // 53-bit uniform in [0, 1): numpy.random.random / random_sample.
  inline double next_double() {
    const uint32_t a = next32() >> 5, b = next32() >> 6;
    return (a * 67108864.0 + b) / 9007199254740992.0;
  }
  // numpy.random.randint(0, n) for 1 <= n: masked rejection sampling on 32-bit
  // draws with mask = the smallest 2^k - 1 >= n - 1; n == 1 draws nothing.
  inline uint32_t bounded(uint32_t n, uint32_t mask) {
    const uint32_t rng = n - 1;
    if (rng == 0) return 0;
    uint32_t v;
    while ((v = (next32() & mask)) > rng) {
    }
    return v;
  }
};

// The generator's position in a local variable for the length of a tight loop:
// the compiler keeps it in a register, where the member would be reloaded after
// every store through the byte arrays the loop fills (they may alias it).  The
// same draws as MT19937's own functions; the position is written back at the end.
struct MTReader {
  MT19937& mt;
  int pos;
  explicit MTReader(MT19937& g) : mt(g), pos(g.pos) {}
  ~MTReader() { mt.pos = pos; }
  inline uint32_t next32() {
    if (pos >= 624) {
      mt.twist();
      pos = 0;
    }
    return mt.out[pos++];
  }
  inline double next_double() {
    const uint32_t a = next32() >> 5, b = next32() >> 6;
    return (a * 67108864.0 + b) / 9007199254740992.0;
  }
  inline uint32_t bounded(uint32_t n, uint32_t mask) {
    const uint32_t rng = n - 1;
    if (rng == 0) return 0;
    uint32_t v;
    while ((v = (next32() & mask)) > rng) {
    }
    return v;
  }
};

static inline uint32_t mask_for(uint32_t n) {
  uint32_t m = n - 1;
  m |= m >> 1;
  m |= m >> 2;
  m |= m >> 4;
  m |= m >> 8;
  m |= m >> 16;
  return m;
}

// The random numbers of a batch of samples.  theboss keeps its input particles in
// a list ordered by mode and pops a uniformly chosen one per step
// (generalized_cliffords_b_simulation_strategy.py:97-105); `idx` holds the
// randint results, i.e. positions in the list of the particles not yet popped.
struct Draws {
  int n = 0;                       // row stride: the most input particles of a sample
  bool binned = false;             // some input mode holds more than one particle
  std::vector<uint8_t> particles;  // [sample][n] particle -> mode of the sample's input (ascending)
  std::vector<uint8_t> nparticles; // [sample] particles of the sample's input
  std::vector<int32_t> L;          // [sample] particles kept
  std::vector<uint8_t> idx;        // [sample][n] randint results
  std::vector<double> u;           // [sample][n] uniforms of numpy.random.choice
  std::vector<uint8_t> modes;      // [sample][n] popped modes (host copy, filled on demand)
};

// Every sample draws from the same input state.
static void same_input(Draws& D, const std::vector<uint8_t>& particles, int n_samples) {
  const int n = (int)particles.size();
  D.n = n;
  D.particles.resize((size_t)n_samples * std::max(n, 1));
  for (int s = 0; s < n_samples; ++s)
    if (n) memcpy(&D.particles[(size_t)s * n], particles.data(), n);
  D.nparticles.assign(n_samples, (uint8_t)n);
}

// The popped modes from the randint results: remove the idx-th remaining particle.
static void modes_from_draws(Draws& D) {
  const int n = D.n, N = (int)D.L.size();
  D.modes.assign((size_t)N * std::max(n, 1), 0);
  uint8_t work[257];
  for (int s = 0; s < N; ++s) {
    const int ns = D.nparticles[s];
    for (int k = 0; k < ns; ++k) work[k] = D.particles[(size_t)s * n + k];
    const uint8_t* is = &D.idx[(size_t)s * n];
    uint8_t* ms = &D.modes[(size_t)s * n];
    for (int k = 0; k < D.L[s]; ++k) {
      const int i = is[k];
      ms[k] = work[i];
      for (int q = 0; q < ns - 1; ++q) work[q] = (q >= i) ? work[q + 1] : work[q];  // fixed trip count
    }
  }
}

// ---------------------------------------------------------------------------
// Parallel replay.  A sample's draws take a data-dependent number of words of
// the MT19937 stream (the particle count from the loss threshold, randint's
// rejections), so the stream's split into samples is sequential by nature.  But
// a parse begun at an arbitrary word meets the true one after a few samples
// (at 20 photons and eta = 0.5: 19 samples on average, at most 141 in 2000
// trials): both are functions of the same words, and from the first sample
// start they share they agree.  So T host threads parse T slices of the
// pre-generated word stream, each from a guessed start; the stitch follows the
// true parse from the stream's start, parses on sequentially across the short
// gap where one slice's parse has not yet met the next one's, and switches to
// the next slice where they meet.  The result is the sequential replay's, word
// for word, and the generator ends in the same state.
// ---------------------------------------------------------------------------

// Host threads for the replay, created on first use and never destroyed (the
// process ends with them parked).  run(T, fn) runs fn(1..T-1) on the pool and
// fn(0) on the caller, and returns when all have finished.  A process forked
// from one with a pool inherits the object but not its threads: its first
// replay makes a pool of its own and leaves the inherited one untouched.
class HostPool {
 public:
  static HostPool& get() {
    static std::atomic<HostPool*> pool{nullptr};
    const pid_t me = getpid();
    HostPool* p = pool.load(std::memory_order_acquire);
    while (!p || p->pid_ != me) {
      HostPool* fresh = new HostPool(me);  // no threads yet: safe to delete if another caller wins
      if (pool.compare_exchange_strong(p, fresh, std::memory_order_acq_rel)) return *fresh;
      delete fresh;
    }
    return *p;
  }
  void run(int T, const std::function<void(int)>& fn) {
    std::lock_guard<std::mutex> serial(run_mu_);
    while (nthreads_ < T - 1) {
      const int id = ++nthreads_;
      std::thread([this, id] { worker(id); }).detach();
    }
    {
      std::lock_guard<std::mutex> lk(mu_);
      fn_ = &fn;
      T_ = T;
      pending_ = T - 1;
      ++epoch_;
    }
    cv_.notify_all();
    fn(0);
    std::unique_lock<std::mutex> lk(mu_);
    done_.wait(lk, [&] { return pending_ == 0; });
  }

 private:
  void worker(int id) {
    uint64_t seen = 0;
    std::unique_lock<std::mutex> lk(mu_);
    for (;;) {
      cv_.wait(lk, [&] { return epoch_ != seen; });
      seen = epoch_;
      if (id < T_) {
        const std::function<void(int)>* f = fn_;
        lk.unlock();
        (*f)(id);
        lk.lock();
        if (--pending_ == 0) done_.notify_one();
      }
    }
  }
  explicit HostPool(pid_t pid) : pid_(pid) {}
  const pid_t pid_;
  std::mutex run_mu_, mu_;
  std::condition_variable cv_, done_;
  const std::function<void(int)>* fn_ = nullptr;
  uint64_t epoch_ = 0;
  int T_ = 0, pending_ = 0, nthreads_ = 0;
};

// The generator's output words from its current state on, with the key of every
// kKeyStride-th block generated, so that the state after any number of words can
// be set (by re-twisting at most kKeyStride - 1 blocks).  The storage is the
// caller's (kept between calls: no page faults on reuse).  One thread generates
// (generate / extend); others may read the words below `ready` (release/acquire)
// while it does.
constexpr uint64_t kKeyStride = 16;
struct WordStream {
  MT19937& mt;
  std::vector<uint32_t>& W;     // the words, in stream order
  std::vector<uint32_t>& keys;  // 624 per kKeyStride generated blocks: the key of blocks 0, 16, ..
  uint32_t key0[624];
  int pos0;
  uint64_t prefix;               // words left in the generator's current block
  uint64_t size = 0;             // words generated
  std::atomic<uint64_t> ready{0};  // words other threads may read
  std::atomic<bool> done{false};   // the parallel phase's generation has ended
  WordStream(MT19937& g, std::vector<uint32_t>& words, std::vector<uint32_t>& block_keys)
      : mt(g), W(words), keys(block_keys), pos0(g.pos) {
    memcpy(key0, g.key, sizeof(key0));
    prefix = (pos0 < 624) ? (uint64_t)(624 - pos0) : 0;
  }
  // Sizes the storage for `words` words and generates them, publishing each block.
  // One more block: its words appended, its key kept when it starts a stride.
  void next_block() {
    const uint64_t k = (size - prefix) / 624;
    mt.twist();
    memcpy(&W[size], mt.out, sizeof(mt.out));
    if (k % kKeyStride == 0) {
      const uint64_t slot = k / kKeyStride;
      if (keys.size() < (slot + 1) * 624) keys.resize((slot + 8) * 624);
      memcpy(&keys[slot * 624], mt.key, sizeof(mt.key));
    }
    size += 624;
  }
  void generate(uint64_t words) {
    const uint64_t blocks = (words > prefix) ? (words - prefix + 623) / 624 : 0;
    if (W.size() < prefix + blocks * 624) W.resize(prefix + blocks * 624);
    if (keys.size() < (blocks / kKeyStride + 1) * 624) keys.resize((blocks / kKeyStride + 1) * 624);
    memcpy(W.data(), mt.out + (pos0 < 624 ? pos0 : 624), sizeof(uint32_t) * prefix);
    size = prefix;
    ready.store(size, std::memory_order_release);
    for (uint64_t k = 0; k < blocks; ++k) {
      next_block();
      ready.store(size, std::memory_order_release);
    }
    done.store(true, std::memory_order_release);
  }
  void extend(uint64_t words) {  // after the parallel phase: at least `words` words
    while (size < words) {
      if (W.size() < size + 624) W.resize(size + 624 * 8);
      next_block();
    }
  }
  // The generator as the sequential replay leaves it after `used` words.
  void finish(uint64_t used) {
    if (used <= prefix) {
      memcpy(mt.key, key0, sizeof(key0));
      mt.pos = pos0 + (int)used;
    } else {
      const uint64_t g = used - prefix, b = (g - 1) / 624;  // block b (0-based) holds the last word used
      const uint64_t b0 = b - b % kKeyStride;
      memcpy(mt.key, &keys[(b0 / kKeyStride) * 624], sizeof(mt.key));
      for (uint64_t q = b0; q < b; ++q) mt.twist_key();
      mt.pos = (int)(g - b * 624);  // in [1, 624]
    }
    if (mt.pos < 624) mt.temper_all();
  }
};

static inline double words_to_double(uint32_t a, uint32_t b) {  // numpy's random_sample from two words
  return ((a >> 5) * 67108864.0 + (b >> 6)) / 9007199254740992.0;
}

struct ReplayParams {
  int n;                  // input particles
  const double* weights;  // particle-number weights (null: every particle kept)
  int nw;
  const uint32_t* masks;  // randint's masks, by particles left
};

// One sample's draws from W[p..avail): 1 done (p advanced), 0 the words ran out
// (p unchanged), -1 the loss threshold lies beyond the weights' sum (theboss's
// randint(low >= high) error; p advanced past the threshold).  The row's
// entries from l on are set to zero.
static inline int parse_sample(const ReplayParams& R, const uint32_t* W, uint64_t avail, uint64_t& p, int32_t& l_out,
                               uint8_t* is, double* us) {
  uint64_t q = p;
  int l = R.n;
  if (R.weights) {  // generalized_cliffords_b_uniform_losses_simulation_strategy.py:67-85
    if (q + 2 > avail) return 0;
    const double thr = words_to_double(W[q], W[q + 1]);
    q += 2;
    double acc = 0.0;
    l = 0;
    for (int i = 0; i < R.nw; ++i) {
      acc += R.weights[i];
      if (acc > thr) break;
      ++l;
    }
    if (l > R.n) {
      p = q;
      l_out = l;
      return -1;
    }
  }
  int remaining = R.n;
  for (int k = 0; k < l; ++k) {  // generalized_cliffords_b_simulation_strategy.py:97-110
    const uint32_t rng = (uint32_t)remaining - 1, mask = R.masks[remaining];
    uint32_t v = 0;
    if (rng) {
      do {
        if (q >= avail) return 0;
        v = W[q++] & mask;
      } while (v > rng);
    }
    is[k] = (uint8_t)v;
    --remaining;
    if (q + 2 > avail) return 0;
    us[k] = words_to_double(W[q], W[q + 1]);
    q += 2;
  }
  for (int k = l; k < R.n; ++k) {
    is[k] = 0;
    us[k] = 0.0;
  }
  p = q;
  l_out = l;
  return 1;
}

// One slice's parse: the samples from word `start` on, until a sample ends at or
// past `stop` or the words run out, in rows of n like the replay's own output.
// The arrays grow as needed and keep their storage between calls; `count`
// records are valid.
struct SliceParse {
  size_t count = 0;
  std::vector<uint64_t> begin, end;
  std::vector<int32_t> L;
  std::vector<uint8_t> idx;  // count x n
  std::vector<double> u;     // count x n
};

static void parse_slice(const ReplayParams& R, WordStream& ws, uint64_t start, uint64_t stop, uint64_t expect_end,
                        double words_per_sample, SliceParse& S) {
  const size_t n = (size_t)std::max(R.n, 1);
  size_t cap = 0;  // records the arrays hold (sized for this call's n: the storage is reused across calls)
  auto grow = [&](size_t c) {
    if (S.begin.size() < c) S.begin.resize(c);
    if (S.end.size() < c) S.end.resize(c);
    if (S.L.size() < c) S.L.resize(c);
    if (S.idx.size() < c * n) S.idx.resize(c * n);
    if (S.u.size() < c * n) S.u.resize(c * n);
    cap = c;
  };
  grow((size_t)((double)(std::min(stop, expect_end) - std::min(start, expect_end)) / std::max(words_per_sample, 1.0) *
               1.1) + 16);
  const uint32_t* W = ws.W.data();  // sized before the parallel phase: stable
  size_t c = 0;
  uint64_t p = start;
  uint64_t avail = ws.ready.load(std::memory_order_acquire);
  while (p < stop) {
    if (c == cap) grow(2 * c + 16);
    int32_t l = 0;
    const uint64_t b = p;
    const int r = parse_sample(R, W, avail, p, l, &S.idx[c * n], &S.u[c * n]);
    if (r == 0) {  // past the generated words: wait for the next block, or stop when generation has ended
      const bool fin = ws.done.load(std::memory_order_acquire);
      const uint64_t now = ws.ready.load(std::memory_order_acquire);
      if (now > avail) {
        avail = now;
        continue;
      }
      if (fin) break;
      std::this_thread::yield();
      continue;
    }
    S.begin[c] = b;
    S.end[c] = p;
    S.L[c] = l;  // l > n marks theboss's error; it matters only on the true parse
    ++c;
  }
  S.count = c;
}

// Expected words per sample (the word buffer's size; a short guess only costs a
// sequential extension at the end).
static double expected_words(const ReplayParams& R) {
  auto kept_words = [&](int l) {
    double w = 0.0;
    for (int k = 0; k < l; ++k) {
      const int r = R.n - k;
      w += 2.0 + (r > 1 ? (double)(R.masks[r] + 1u) / r : 0.0);
    }
    return w;
  };
  if (!R.weights) return kept_words(R.n);
  double e = 2.0, tot = 0.0;
  for (int l = 0; l <= R.n && l < R.nw; ++l) tot += std::max(R.weights[l], 0.0);
  for (int l = 0; l <= R.n && l < R.nw; ++l) e += std::max(R.weights[l], 0.0) / (tot > 0 ? tot : 1.0) * kept_words(l);
  return e;
}

struct ReplayScratch {
  std::vector<uint32_t> W, keys;
  std::vector<SliceParse> S;
};

// The parallel replay of N samples into L (N), idx and u (N x n).  The calling
// thread generates the words while T pool threads parse the T slices, each
// following the words as they appear; then the calling thread stitches.
static int replay_parallel(const ReplayParams& R, MT19937& mt, int N, int T, int32_t* L, uint8_t* idx, double* u) {
  const size_t n = (size_t)std::max(R.n, 1);
  static thread_local ReplayScratch rs;  // the calling thread's, reused
  const double ew = expected_words(R);
  const uint64_t est = (uint64_t)(N * ew * 1.03) + 4096;
  WordStream ws(mt, rs.W, rs.keys);
  std::vector<uint64_t> cut(T + 1);
  for (int t = 0; t <= T; ++t) cut[t] = est * (uint64_t)t / (uint64_t)T;
  if ((int)rs.S.size() < T) rs.S.resize(T);
  std::vector<SliceParse>& S = rs.S;
  {
    // storage sized before any reader starts; generate() only writes into it
    const uint64_t blocks = (est > ws.prefix) ? (est - ws.prefix + 623) / 624 : 0;
    if (rs.W.size() < ws.prefix + blocks * 624) rs.W.resize(ws.prefix + blocks * 624);
  }
  HostPool::get().run(T + 1, [&](int t) {
    if (t == 0)
      ws.generate(est);
    else
      parse_slice(R, ws, cut[t - 1], t < T ? cut[t] : UINT64_MAX, est, ew, S[t - 1]);
  });
  // stitch: follow the true parse from word 0
  int count = 0;
  uint64_t p = 0;
  bool failed = false;  // theboss's randint error on the true parse
  auto sequential = [&]() {  // one sample parsed at p, extending the words as needed
    for (;;) {
      int32_t l = 0;
      const int r = parse_sample(R, ws.W.data(), ws.size, p, l, idx + (size_t)count * n, u + (size_t)count * n);
      if (r < 0) {
        failed = true;
        return;
      }
      if (r > 0) {
        L[count++] = l;
        return;
      }
      ws.extend(ws.size + 624 * 8);
    }
  };
  for (int t = 0; t < T && count < N && !failed; ++t) {
    const SliceParse& P = S[t];
    const size_t cnt = P.count;
    size_t j = std::lower_bound(P.begin.begin(), P.begin.begin() + cnt, p) - P.begin.begin();
    while (count < N && !failed && j < cnt && P.begin[j] != p) {  // not met yet: parse across the gap
      sequential();
      while (j < cnt && P.begin[j] < p) ++j;
    }
    if (failed || j >= cnt || P.begin[j] != p || count >= N) continue;
    // from row j on the slice's parse is the true one: copy its rows in one piece
    size_t j1 = std::min(cnt, j + (size_t)(N - count));
    for (size_t q = j; q < j1; ++q)
      if (P.L[q] > R.n) {  // theboss's error on the true parse: rows before it stand
        j1 = q;
        failed = true;
        break;
      }
    memcpy(L + count, &P.L[j], sizeof(int32_t) * (j1 - j));
    memcpy(idx + (size_t)count * n, &P.idx[j * n], (j1 - j) * n);
    memcpy(u + (size_t)count * n, &P.u[j * n], sizeof(double) * (j1 - j) * n);
    count += (int)(j1 - j);
    p = failed ? P.end[j1] : P.end[j1 - 1];
  }
  while (count < N && !failed) sequential();
  ws.finish(p);
  if (failed) {
    set_error("randint: low >= high (particle-number weights sum below the threshold)");
    return kErrArg;
  }
  return kOk;
}

// Host threads for a replay of N samples: one per 512 samples, at most 8 and at
// most half the host's hardware threads; 1 means the sequential replay.
static int replay_threads(int N, int n) {
  if (n < 1 || N < 1024) return 1;
  const int hw = (int)std::thread::hardware_concurrency();
  return std::max(1, std::min({8, N / 512, hw > 1 ? hw / 2 : 1}));
}

// The whole random stream of `n_samples` GC&C-B samples, in theboss's draw order.
static int predraw(const int32_t* input_state, int m, const double* weights, int n_weights, MT19937& mt,
                   int n_samples, Draws& D) {
  if (m > 256) {
    set_error("the sampler supports at most 256 modes");
    return kErrLimit;
  }
  int n = 0;
  D.binned = false;
  for (int i = 0; i < m; ++i) {
    if (input_state[i] < 0 || input_state[i] > 255) {
      set_error("input occupations must be in [0, 255]");
      return kErrArg;
    }
    if (input_state[i] > 1) D.binned = true;
    n += input_state[i];
  }
  if (n > 255) {
    set_error("at most 255 input particles");
    return kErrLimit;
  }
  {
    std::vector<uint8_t> particles;
    for (int i = 0; i < m; ++i)
      for (int k = 0; k < input_state[i]; ++k) particles.push_back((uint8_t)i);
    same_input(D, particles, n_samples);
  }
  if (weights && n_weights != n + 1) {
    set_error("particle-number weights must have n + 1 entries");
    return kErrArg;
  }
  std::vector<int32_t>& L = D.L;
  L.assign(n_samples, 0);
  D.idx.assign((size_t)n_samples * std::max(n, 1), 0);
  D.u.assign((size_t)n_samples * std::max(n, 1), 0.0);
  D.modes.clear();
  uint32_t masks[257];
  for (int r = 1; r <= n; ++r) masks[r] = mask_for((uint32_t)r);
  const int T = replay_threads(n_samples, n);
  if (T > 1) {
    const ReplayParams R{n, weights, n_weights, masks};
    return replay_parallel(R, mt, n_samples, T, L.data(), D.idx.data(), D.u.data());
  }
  MTReader rd(mt);
  for (int s = 0; s < n_samples; ++s) {
    int l = n;
    if (weights) {  // generalized_cliffords_b_uniform_losses_simulation_strategy.py:67-85
      const double thr = rd.next_double();
      double acc = 0.0;
      l = 0;
      for (int i = 0; i < n_weights; ++i) {
        acc += weights[i];
        if (acc > thr) break;
        ++l;
      }
      if (l > n) {
        set_error("randint: low >= high (particle-number weights sum below the threshold)");
        return kErrArg;
      }
    }
    L[s] = l;
    int remaining = n;
    uint8_t* is = &D.idx[(size_t)s * n];
    double* us = &D.u[(size_t)s * n];
    for (int k = 0; k < l; ++k) {  // generalized_cliffords_b_simulation_strategy.py:97-110
      is[k] = (uint8_t)rd.bounded((uint32_t)remaining, masks[remaining]);
      --remaining;
      us[k] = rd.next_double();
    }
  }
  return kOk;
}

// ---------------------------------------------------------------------------
// Device side
// ---------------------------------------------------------------------------
struct LevelSample {  // host-computed layout of one sample's sweep at one level
  int64_t n_codes;
  int64_t thread_begin;
  int64_t n_threads;
  int64_t part_off;
  int64_t pool_off;
};

struct FinalizeArgs {
  int k;       // level = input particles of this step
  int A;       // active samples at this level
  int A_next;  // active samples at level k + 1
  int m;
  int n;       // row stride of idx / uni
  int fx;      // fixed-point fraction bits of the sweep rows
  const longlong2* Ufx;   // m x m, U * 2^fx rounded
  const float4* Uff;      // float-pair pmf: m x m transposed, Uff[i * m + o] = U[o][i] as float pairs
                          // (re hi, re lo, im hi, im lo)
  const int4* Ulimb;      // FP64 pmf: m x m transposed, U[o][i] * 2^lfx rounded, as 27-bit limbs
                          // (re lo, re hi, im lo, im hi; lo in [0, 2^27), value = hi 2^27 + lo)
  int lfx;                // |U| * 2^lfx < 2^53
  const float* Uabs;      // m x m transposed, |Re U[o][i]| + |Im U[o][i]| (the pmf error bound)
  uint8_t* S;             // [sample][m] current input occupations
  uint8_t* T;             // [sample][m] output occupations
  const int32_t* order;   // [sample in level order] -> its row in the replayed (input-order) draws
  const uint8_t* idx;     // [input-order sample][n] randint results (position among the particles left)
  const uint8_t* pmode;   // [input-order sample][n] particle -> input mode
  const uint8_t* npart;   // [input-order sample] input particles
  int64_t mstride;        // elements between the samples' matrices (0: one matrix for all)
  uint32_t* rem;          // [sample][8] particles not yet popped, as bits
  const double* uni;      // [input-order sample][n] uniforms
  const SweepProblem* probs_cur;
  const uint8_t* dmode_cur;  // [sample][32]
  const double2* partials;
  const double2* reduced;       // FP64 levels with long partial sums: the sums, 32 per sample (else null)
  SweepProblem* probs_next;
  uint8_t* dmode_next;
  longlong2* pool_next;
  const LevelSample* next_tab;  // A_next entries, or null when the next level is uniform
  LevelSample next_uni;         // uniform next level: n_codes, threads per sample and the per-sample
                                // strides of partials (part_off) and rows (pool_off)
  int next_group;               // uniform next level: threads per summed group of minors
  int cur_ff;                   // this level's sweep ran on float pairs: its partials are float4
  int next_ff;                  // the next level's sweep runs on float pairs (float-pair rows, biases)
  int* err;                     // err[0]: a pmf could not be normalised; err[1]: draws decided by the
                                // exact sequential rule because a cdf step lay within the error window
};

constexpr int kFinWarps = 4;

// Stated relative error bounds of the all-minors sweeps (absolute error of every
// minor against the exact value, over the largest minor of the step), used by the
// finalize kernel's cdf guard.  Measured against the double-double oracle at
// k = 8..22 input particles: FP64 sweeps at most 8.1e-15, float-pair sweeps at
// most 3.0e-12; the bounds hold 110x and 19x of margin.
constexpr float kMinorsErrF64 = 9.094947e-13f;  // 2^-40
constexpr float kMinorsErrFF = 5.820766e-11f;   // 2^-34

__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long y = __shfl_xor_sync(0xffffffffu, v, o);
    v = y > v ? y : v;
  }
  return v;
}

__device__ __forceinline__ float warp_sum_f(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// x * 2^s in float for |s| <= 252 (two exact power-of-two factors; the product
// over- or underflows like any float product).
__device__ __forceinline__ float scale_pow2f(float x, int s) {
  s = max(-252, min(s, 252));
  const int h = s / 2, l = s - h;
  return x * __int_as_float((h + 127) << 23) * __int_as_float((l + 127) << 23);
}

// x * 2^F rounded to the nearest integer (ties up), for a finite x >= 0 with
// x * 2^F < 2^63; integer instructions only (the double's fields are shifted).
__device__ __forceinline__ unsigned long long fixed_of_double(double x, int F) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int e = (int)(b >> 52) & 0x7ff;
  unsigned long long mant = b & 0xFFFFFFFFFFFFFull;
  if (e) mant |= 1ull << 52;
  const int sh = (e ? e : 1) - 1075 + F;  // x = mant * 2^((e ? e : 1) - 1075)
  if (sh >= 0) return mant << sh;         // the caller keeps x * 2^F below 2^63
  if (sh <= -64) return 0ull;
  return (mant >> -sh) + ((mant >> (-sh - 1)) & 1ull);
}

// Removes the r-th (0-based) particle still in a 256-bit set held one 32-bit word
// per lane (lanes 0..7, the rest 0; r is below the set's size: the host drew it
// with randint(0, remaining)).  Every lane gets the particle's index; the owning
// lane's word loses its bit.
__device__ __forceinline__ int pop_particle_warp(uint32_t& remw, int r, int lane) {
  const int c = (lane < 8) ? __popc(remw) : 0;
  int incl = c;  // inclusive prefix over the words
#pragma unroll
  for (int off = 1; off < 8; off <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, incl, off);
    if (lane >= off) incl += y;
  }
  const int excl = incl - c;
  const unsigned who = __ballot_sync(0xffffffffu, lane < 8 && r >= excl && r < incl);
  const int q = __ffs(who) - 1;  // the word holding it (r is below the set's size: the host drew it)
  int pos = 0;
  if (lane == q) {
    int rr = r - excl;
    uint32_t x = remw;
    for (int s = 16; s > 0; s >>= 1) {  // binary search for the bit
      const uint32_t lo = x & ((1u << s) - 1u);
      const int cl = __popc(lo);
      if (rr >= cl) {
        rr -= cl;
        x >>= s;
        pos += s;
      } else {
        x = lo;
      }
    }
    remw &= ~(1u << pos);
  }
  return q * 32 + __shfl_sync(0xffffffffu, pos, q);
}

// (r2 2^54 + r1 2^27 + r0) 2^e rounded to the nearest double (ties to even), in
// integer instructions: the three 64-bit sums of the exact Laplace step (|sum| <
// 2^113) combined in 128 bits, normalised by a leading-zero count, rounded once.
// The exponent is folded in when the result is a normal double; otherwise the
// rounded value is scaled by ldexp (exact unless it under- or overflows).
__device__ __forceinline__ double limbs_to_double(long long r2, long long r1, long long r0, int e) {
  // 128-bit two's complement value hi:lo
  unsigned long long lo = (unsigned long long)r2 << 54;
  long long hi = r2 >> 10;
  const unsigned long long l1 = (unsigned long long)r1 << 27;
  const unsigned long long s1 = lo + l1;
  hi += (r1 >> 37) + (s1 < lo ? 1 : 0);
  const unsigned long long s2 = s1 + (unsigned long long)r0;
  hi += (r0 >> 63) + (s2 < s1 ? 1 : 0);
  lo = s2;
  const bool neg = hi < 0;
  unsigned long long mh = (unsigned long long)hi, ml = lo;
  if (neg) {  // magnitude
    ml = ~ml + 1ull;
    mh = ~mh + (ml == 0 ? 1ull : 0ull);
  }
  if ((mh | ml) == 0) return 0.0;
  const int lz = mh ? __clzll((long long)mh) : 64 + __clzll((long long)ml);
  unsigned long long th, tl;  // the magnitude shifted left by lz: its top bit at bit 127
  if (lz >= 64) {
    th = ml << (lz - 64);
    tl = 0;
  } else if (lz == 0) {
    th = mh;
    tl = ml;
  } else {
    th = (mh << lz) | (ml >> (64 - lz));
    tl = ml << lz;
  }
  unsigned long long m = th >> 11;  // 53 bits
  const unsigned long long rem = th & 0x7FFull;
  if (rem > 0x400ull || (rem == 0x400ull && (tl != 0 || (m & 1ull)))) m += 1ull;
  int ex = 127 - lz;  // |value| = m 2^(ex - 52)
  if (m >> 53) {
    m >>= 1;
    ++ex;
  }
  const int be = ex + e + 1023;
  const unsigned long long sign = neg ? (1ull << 63) : 0ull;
  if (be >= 1 && be <= 2046)
    return __longlong_as_double((long long)(sign | ((unsigned long long)be << 52) | (m & 0xFFFFFFFFFFFFFull)));
  const double v = __longlong_as_double((long long)(sign | ((unsigned long long)(ex + 1023) << 52) | (m & 0xFFFFFFFFFFFFFull)));
  return ldexp(v, e);
}

// The levels where each sample's sweep leaves many partial rows (the top levels:
// a few samples, thousands of threads each) sum them here, one block of 128
// threads per (sample, digit), instead of in the finalize's single warp, whose
// dependent loads and adds made that sum its slowest phase.  Thread t adds rows
// t, t + 128, .. in order, then a fixed-order tree; the result is unscaled
// (the finalize applies the problem's scale), row j of `out` holds sample j's
// digits.
constexpr int kReduceMinParts = 32;   // partial rows per sample from which a level gets this kernel,
constexpr int kReduceMaxSamples = 16; // when it has this many samples at most (at the level with 1297
                                      // samples and 45 rows each it cost 64 us against the finalize's
                                      // own few microseconds of summing)
__global__ void __launch_bounds__(128) gccb_partials_reduce_kernel(const SweepProblem* __restrict__ probs,
                                                                  const double2* __restrict__ partials,
                                                                  double2* __restrict__ out) {
  __shared__ double sx[128], sy[128];
  const int j = blockIdx.x, d = blockIdx.y;
  const SweepProblem& P = probs[j];
  const int nd = P.nd + P.fixed_digit;
  if (d >= nd) return;
  const int64_t parts = P.n_threads / P.group;
  double x = 0.0, y = 0.0;
#pragma unroll 4
  for (int64_t q = threadIdx.x; q < parts; q += 128) {
    const double2 v = partials[P.part_off + q * nd + d];
    x += v.x;
    y += v.y;
  }
  sx[threadIdx.x] = x;
  sy[threadIdx.x] = y;
  __syncthreads();
  for (int h = 64; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h) {
      sx[threadIdx.x] += sx[threadIdx.x + h];
      sy[threadIdx.x] += sy[threadIdx.x + h];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) out[(size_t)j * 32 + d] = make_double2(sx[0], sy[0]);
}

// kF64: the minors, the Laplace step, |.|^2 and the pmf are FP64 (the default);
// otherwise float pairs on the FP32 pipe (the opt-in float-pair arithmetic).
template <bool kF64>
__global__ void __launch_bounds__(kFinWarps * 32, 8) gccb_finalize_kernel(FinalizeArgs a) {
  __shared__ double2 sub_s[kFinWarps][32];
  __shared__ float4 subf_s[kFinWarps][32];
  __shared__ uint8_t dm_s[kFinWarps][32];
  __shared__ uint8_t mult_s[kFinWarps][32];
  __shared__ uint8_t fm_s[kFinWarps][32];
  __shared__ double pmf_s[kFinWarps][256];
  __shared__ float cn_s[kFinWarps][32];  // |c_d|_1 2^-Ec (the pmf error bound)
  __shared__ int4 climb_s[kFinWarps][32];  // FP64 pmf: the minors as 27-bit limbs (re lo, re hi, im lo, im hi)
  __shared__ int2 cnb_s[kFinWarps][32];    // and -Im as limbs
  __shared__ uint8_t srow_s[kFinWarps][256];  // the sample's input and output occupations, kept here
  __shared__ uint8_t trow_s[kFinWarps][256];  // while the kernel updates them (written through to S, T)
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int j = blockIdx.x * kFinWarps + w;
  if (j >= a.A) return;
  const int m = a.m;
  const longlong2* Ufxs = a.Ufx + (size_t)j * a.mstride;  // and its fixed-point copy
  uint8_t* S = a.S + (size_t)j * m;
  uint8_t* T = a.T + (size_t)j * m;
  // Everything the particle bookkeeping needs, loaded up front (independent
  // loads, in flight during the sums below): the occupations, the sample's
  // randint results and particle modes (one per lane; at most 32 particles), and
  // its set of particles not yet popped (one word per lane 0..7).
  const size_t drow = (size_t)a.order[j] * a.n;  // this sample's replayed draws
  for (int i = lane; i < m; i += 32) {
    srow_s[w][i] = S[i];
    trow_s[w][i] = T[i];
  }
  const int idxv = (lane < a.n) ? (int)a.idx[drow + lane] : 0;
  const int pmv = (lane < a.n) ? (int)a.pmode[drow + lane] : 0;
  uint32_t remw = 0;
  if (a.k == 1) {
    const int np = a.npart[a.order[j]];
    const int lo = lane * 32;
    if (lane < 8) remw = (np >= lo + 32) ? 0xffffffffu : (np > lo ? ((1u << (np - lo)) - 1u) : 0u);
  } else if (lane < 8) {
    remw = a.rem[(size_t)j * 8 + lane];
  }
  __syncwarp();
  int nd;
  if (a.k == 1) {
    // one particle: the minors are the input occupations themselves
    // (bs_submatrices_permanent_calculator_base.py:157-158)
    const int mode = __shfl_sync(0xffffffffu, pmv, pop_particle_warp(remw, __shfl_sync(0xffffffffu, idxv, 0), lane));
    if (lane == 0) {
      srow_s[w][mode] = 1;
      S[mode] = 1;
      subf_s[w][0] = make_float4(1.0f, 0.0f, 0.0f, 0.0f);
      sub_s[w][0] = make_double2(1.0, 0.0);
      dm_s[w][0] = (uint8_t)mode;
      mult_s[w][0] = 1;
    }
    nd = 1;
  } else {
    const SweepProblem& P = a.probs_cur[j];
    nd = P.nd + P.fixed_digit;  // the held (halved) digit's minor is the last row
    const int64_t parts = P.n_threads / P.group;
    if (a.cur_ff) {
      // float-pair partials: summed as float pairs in a fixed order, scaled by the
      // problem's power of two, exactly in float when that power is a normal float
      // (always, for factors of comparable size); otherwise in FP64 below
      const float4* fp = reinterpret_cast<const float4*>(a.partials) + P.part_off;
      const int sc_exp = (int)((__double_as_longlong(P.scale) >> 52) & 0x7FF) - 1023;
      const bool sc_float = sc_exp >= -126 && sc_exp <= 127;
      const float sc = sc_float ? __double2float_rn(P.scale) : 1.0f;
      if (parts <= 64) {
        if (lane < nd) {
          float rh = 0.0f, rl = 0.0f, ih = 0.0f, il = 0.0f;
#pragma unroll 8
          for (int64_t q = 0; q < parts; ++q) {  // unrolled: 8 loads in flight
            const float4 v = fp[q * nd + lane];
            ff_acc(rh, rl, 1.0f, v.x, v.y);
            ff_acc(ih, il, 1.0f, v.z, v.w);
          }
          subf_s[w][lane] = make_float4(rh * sc, rl * sc, ih * sc, il * sc);
        }
      } else {
        for (int d = 0; d < nd; ++d) {
          float rh = 0.0f, rl = 0.0f, ih = 0.0f, il = 0.0f;
          for (int64_t q = lane; q < parts; q += 32) {
            const float4 v = fp[q * nd + d];
            ff_acc(rh, rl, 1.0f, v.x, v.y);
            ff_acc(ih, il, 1.0f, v.z, v.w);
          }
#pragma unroll
          for (int off = 16; off > 0; off >>= 1) {  // fixed butterfly order
            const float orh = __shfl_xor_sync(0xffffffffu, rh, off), orl = __shfl_xor_sync(0xffffffffu, rl, off);
            const float oih = __shfl_xor_sync(0xffffffffu, ih, off), oil = __shfl_xor_sync(0xffffffffu, il, off);
            ff_acc(rh, rl, 1.0f, orh, orl);
            ff_acc(ih, il, 1.0f, oih, oil);
          }
          if (lane == d) subf_s[w][d] = make_float4(rh * sc, rl * sc, ih * sc, il * sc);
        }
      }
    } else if (a.reduced) {  // summed by gccb_partials_reduce_kernel
      if (lane < nd) {
        const double2 v = a.reduced[(size_t)j * 32 + lane];
        sub_s[w][lane] = make_double2(v.x * P.scale, v.y * P.scale);
      }
    } else {
      // FP64 partials (parts x nd), summed in a fixed order.  Every FP64
      // instruction holds the pipe for a whole warp however few lanes are active,
      // so the lanes are spread over the partials: either gc <= 32 / nd groups of
      // nd lanes (lane g * nd + d sums rows g, g + gc, .. of digit d, then lane d
      // adds up the gc group sums; gc = 1 is one lane per digit), or, with many
      // partials, all 32 lanes stripe over each digit's rows and a butterfly sums
      // them; whichever issues fewer FP64 instructions.
      int gc = 1;
      int64_t cost_groups = 2 * (parts - 1);  // each group's first row is a copy, not an add
      for (int g2 = 2; g2 * nd <= 32 && g2 <= parts; ++g2) {
        const int64_t c = 2 * ((parts + g2 - 1) / g2 - 1) + 2 * (g2 - 1);
        if (c < cost_groups) {
          cost_groups = c;
          gc = g2;
        }
      }
      const int64_t cost_stripes = (int64_t)nd * (2 * ((parts + 31) / 32) + 10);
      if (cost_groups <= cost_stripes) {
        const int g = lane / nd, d = lane - g * nd;
        double sx = 0.0, sy = 0.0;
        if (g < gc && parts >= 8 * gc) {
          // long sums (the top levels, where one warp has the SM's FP64 unit to
          // itself): four interleaved chains, rows g + (4 i + c) gc in chain c,
          // combined in a fixed order, a quarter of one chain's latency
          double x0 = 0.0, y0 = 0.0, x1 = 0.0, y1 = 0.0, x2 = 0.0, y2 = 0.0, x3 = 0.0, y3 = 0.0;
          int64_t q = g;
#pragma unroll 4
          for (; q + 3 * gc < parts; q += 4 * gc) {
            const double2 v0 = a.partials[P.part_off + q * nd + d];
            const double2 v1 = a.partials[P.part_off + (q + gc) * nd + d];
            const double2 v2 = a.partials[P.part_off + (q + 2 * gc) * nd + d];
            const double2 v3 = a.partials[P.part_off + (q + 3 * gc) * nd + d];
            x0 += v0.x;
            y0 += v0.y;
            x1 += v1.x;
            y1 += v1.y;
            x2 += v2.x;
            y2 += v2.y;
            x3 += v3.x;
            y3 += v3.y;
          }
          for (; q < parts; q += gc) {
            const double2 v = a.partials[P.part_off + q * nd + d];
            x0 += v.x;
            y0 += v.y;
          }
          sx = (x0 + x1) + (x2 + x3);
          sy = (y0 + y1) + (y2 + y3);
        } else if (g < gc) {  // gc <= parts: every group has a first row
          const double2 v0 = a.partials[P.part_off + (int64_t)g * nd + d];
          sx = v0.x;
          sy = v0.y;
#pragma unroll 8
          for (int64_t q = g + gc; q < parts; q += gc) {
            const double2 v = a.partials[P.part_off + q * nd + d];
            sx += v.x;
            sy += v.y;
          }
        }
        sub_s[w][lane] = make_double2(sx, sy);
        __syncwarp();
        if (lane < nd) {
          double tx = sx, ty = sy;  // group 0 is this lane's own sum
          for (int gg = 1; gg < gc; ++gg) {
            const double2 v = sub_s[w][gg * nd + lane];
            tx += v.x;
            ty += v.y;
          }
          sx = tx * P.scale;
          sy = ty * P.scale;
        }
        __syncwarp();
        if (lane < nd) sub_s[w][lane] = make_double2(sx, sy);
      } else {  // many partials: the lanes stripe over them, then a fixed-order warp
                // sum; two digits at a time (independent chains in flight)
        for (int d = 0; d < nd; d += 2) {
          const int d1 = (d + 1 < nd) ? d + 1 : d;  // an odd last digit is summed twice, stored once
          double sx = 0.0, sy = 0.0, tx = 0.0, ty = 0.0;
#pragma unroll 4
          for (int64_t q = lane; q < parts; q += 32) {
            const double2 v = a.partials[P.part_off + q * nd + d];
            const double2 u = a.partials[P.part_off + q * nd + d1];
            sx += v.x;
            sy += v.y;
            tx += u.x;
            ty += u.y;
          }
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) {  // warp_sum's butterfly, the four sums interleaved
            sx += __shfl_xor_sync(0xffffffffu, sx, o);
            sy += __shfl_xor_sync(0xffffffffu, sy, o);
            tx += __shfl_xor_sync(0xffffffffu, tx, o);
            ty += __shfl_xor_sync(0xffffffffu, ty, o);
          }
          if (lane == d) sub_s[w][d] = make_double2(sx * P.scale, sy * P.scale);
          if (lane == d1 && d1 != d) sub_s[w][d1] = make_double2(tx * P.scale, ty * P.scale);
        }
      }
    }
    if (lane < nd) {
      dm_s[w][lane] = a.dmode_cur[(size_t)j * 32 + lane];
      mult_s[w][lane] = P.mult[lane];
    }
  }
  __syncwarp();
  const double uu = a.uni[drow + (a.k - 1)];
  const int K = (m + 31) >> 5;  // contiguous outputs per lane in the cdf scan
  const int o0 = lane * K;
  const int full = m & ~31;
  int idx = 0;
  bool near = false;  // some cdf step lies within the error window of u * total
  // theboss: Laplace expansion perm(T + e_o) = sum_i S_i sub_i U[o][i], |.|^2,
  // normalisation by Python's sequential sum
  // (generalized_cliffords_b_simulation_strategy.py:82-92), then numpy.random.choice:
  // cdf = cumsum(p), cdf /= cdf[-1], searchsorted(cdf, u, 'right') (:107-110).  The
  // Glynn-form sweep already delivers S_i sub_i.  Lane o reads column o of the
  // transposed matrix (coalesced); the outputs that do not fill a warp split their
  // digits over several lanes.
  //
  // Fast path: the decision from a scan of the unnormalised pmf compared with
  // u * total (no division).  The cdf guard: with c_d the minors, a_o =
  // sum_d |c_d| |U[o][d]| and b_o = sum_d |U[o][d]| (1-norms of the complex
  // entries, upper bounds), each minor is within eps_m * max_d |c_d| of its exact
  // value (kMinorsErrF64 / kMinorsErrFF), so |p_o - exact| <= e_o = eps_m max|c| b_o
  // + gamma a_o and |pmf_o - exact| <= e_o (2 a_o + e_o) (|p_o| <= a_o).  Their sum E
  // plus the scan's and theboss's own rounding of the sums bounds how far every
  // cdf step can lie from the exact one.  When a step lies within that window of
  // u * total the draw is decided by theboss's exact sequential rule on the pmf
  // and counted in err[1]; outside it the fast path's decision is the exact one.
  if constexpr (kF64) {
    // ---- FP64 pmf (the default arithmetic) ----
    // The Laplace sums are exact: the minors (scaled by 2^(52 - Ec), Ec their
    // largest 1-norm's exponent) and U (scaled by 2^lfx) are rounded once to
    // integers below 2^53, split into 27-bit limbs (x = x1 2^27 + x0, x0 >= 0),
    // and every limb product (below 2^54) is added into three 64-bit sums per
    // component (the 2^54, 2^27 and 2^0 parts; at most 4 nd <= 128 products each,
    // no overflow).  Those sums are combined in 128 bits and rounded once to a
    // double.  The products run on the integer pipe (a 32 x 32 -> 64-bit
    // multiply-add each, 16 per digit and output), which GB300 issues far faster
    // than its FP64 pipe; only |.|^2 (2 DFMA per output) stays on the FP64 pipe.
    const int4* UL = a.Ulimb + (size_t)j * a.mstride;
    const float* UA = a.Uabs + (size_t)j * a.mstride;
    double* pmf = pmf_s[w];
    // the bound's scale: 2^-Ec, 2^Ec <= max_d |c_d|_1 < 2^(Ec + 1)
    double c1 = 0.0;
    double2 cv = make_double2(0.0, 0.0);
    if (lane < nd) {
      cv = sub_s[w][lane];
      c1 = fabs(cv.x) + fabs(cv.y);
    }
    const unsigned long long cb = warp_max_u64((unsigned long long)__double_as_longlong(c1));
    const int Ec = (int)(cb >> 52) - 1023;  // non-negative doubles order as integers
    const double sc = (cb >> 52) ? __longlong_as_double((long long)(1023 - Ec) << 52) : 1.0;  // 2^-Ec
    float cn = 0.0f;
    if (lane < nd) {
      cn = __double2float_ru(c1 * sc);  // in [0, 2)
      cn_s[w][lane] = cn;
      // c * 2^(52 - Ec) (exact: a power of two; every component < 2^53), rounded
      const double s52 = sc * 4503599627370496.0;  // 2^52
      const long long A = __double2ll_rn(cv.x * s52), B = __double2ll_rn(cv.y * s52);
      const long long NB = -B;
      climb_s[w][lane] = make_int4((int)(A & 0x7FFFFFF), (int)(A >> 27), (int)(B & 0x7FFFFFF), (int)(B >> 27));
      cnb_s[w][lane] = make_int2((int)(NB & 0x7FFFFFF), (int)(NB >> 27));
    }
    const float csum = warp_sum_f(cn);  // sum_d |c_d|_1 2^-Ec
    __syncwarp();
    // e_o in units of 2^Ec: the minors' error, the rounding of c (half a unit of
    // 2^(Ec - 52) per component) and of U (half a unit of 2^-lfx) to integers, and
    // the rounding of the exact sum to a double, each counted twice
    const float ec_b = 2.0f * kMinorsErrF64 + 4.440892e-16f;  // times b_o: eps_m max|c| + 2 2^-52
    const float ec_c = scale_pow2f(csum, 1 - a.lfx);            // 2^(1 - lfx) sum_d |c_d|_1
    const float ec_a = 2.220446e-16f;                           // times a_o: 2 2^-53
    const int pexp = Ec - 52 - a.lfx;                          // the sums' unit: 2^pexp
    float errsum = 0.0f;                                        // this lane's share of E * 2^-2Ec
    for (int o = lane; o < full; o += 32) {
      long long r2 = 0, r1 = 0, r0 = 0, i2 = 0, i1 = 0, i0 = 0;
      float ao = 0.0f, bo = 0.0f;
#pragma unroll 8  // independent gathers in flight
      for (int d = 0; d < nd; ++d) {
        const int4 c = climb_s[w][d];  // a0 a1 b0 b1
        const int2 nb = cnb_s[w][d];   // (-b)0 (-b)1
        const int e = dm_s[w][d] * m + o;
        const int4 u = UL[e];          // x0 x1 y0 y1
        const float ua = UA[e];
        r2 += (long long)c.y * u.y + (long long)nb.y * u.w;
        r1 += (long long)c.y * u.x + (long long)c.x * u.y + (long long)nb.y * u.z + (long long)nb.x * u.w;
        r0 += (long long)c.x * u.x + (long long)nb.x * u.z;
        i2 += (long long)c.y * u.w + (long long)c.w * u.y;
        i1 += (long long)c.y * u.z + (long long)c.x * u.w + (long long)c.w * u.x + (long long)c.z * u.y;
        i0 += (long long)c.x * u.z + (long long)c.z * u.x;
        ao = fmaf(cn_s[w][d], ua, ao);
        bo += ua;
      }
      const double pr = limbs_to_double(r2, r1, r0, pexp);
      const double pi = limbs_to_double(i2, i1, i0, pexp);
      pmf[o] = fma(pr, pr, pi * pi);
      const float eo = ec_b * bo + ec_c + ec_a * ao;
      errsum += eo * (2.0f * ao + eo) + 4.440892e-16f * ao * ao;  // + |.|^2's two roundings
    }
    if (m > full) {
      const int r = m - full;
      int s = 1;  // lanes per remaining output (a power of two, r * s <= 32)
      while (r * (s << 1) <= 32) s <<= 1;
      const int oi = lane / s, c0 = lane & (s - 1);
      long long r2 = 0, r1 = 0, r0 = 0, i2 = 0, i1 = 0, i0 = 0;
      float ao = 0.0f, bo = 0.0f;
      if (oi < r) {
#pragma unroll 4
        for (int d = c0; d < nd; d += s) {
          const int4 c = climb_s[w][d];
          const int2 nb = cnb_s[w][d];
          const int e = dm_s[w][d] * m + full + oi;
          const int4 u = UL[e];
          const float ua = UA[e];
          r2 += (long long)c.y * u.y + (long long)nb.y * u.w;
          r1 += (long long)c.y * u.x + (long long)c.x * u.y + (long long)nb.y * u.z + (long long)nb.x * u.w;
          r0 += (long long)c.x * u.x + (long long)nb.x * u.z;
          i2 += (long long)c.y * u.w + (long long)c.w * u.y;
          i1 += (long long)c.y * u.z + (long long)c.x * u.w + (long long)c.w * u.x + (long long)c.z * u.y;
          i0 += (long long)c.x * u.z + (long long)c.z * u.x;
          ao = fmaf(cn_s[w][d], ua, ao);
          bo += ua;
        }
      }
      for (int off = s >> 1; off > 0; off >>= 1) {  // the output's lanes: exact integer sums
        r2 += __shfl_xor_sync(0xffffffffu, r2, off);
        r1 += __shfl_xor_sync(0xffffffffu, r1, off);
        r0 += __shfl_xor_sync(0xffffffffu, r0, off);
        i2 += __shfl_xor_sync(0xffffffffu, i2, off);
        i1 += __shfl_xor_sync(0xffffffffu, i1, off);
        i0 += __shfl_xor_sync(0xffffffffu, i0, off);
        ao += __shfl_xor_sync(0xffffffffu, ao, off);
        bo += __shfl_xor_sync(0xffffffffu, bo, off);
      }
      if (oi < r && c0 == 0) {
        const double pr = limbs_to_double(r2, r1, r0, pexp);
        const double pi = limbs_to_double(i2, i1, i0, pexp);
        pmf[full + oi] = fma(pr, pr, pi * pi);
        const float eo = ec_b * bo + ec_c + ec_a * ao;
        errsum += eo * (2.0f * ao + eo) + 4.440892e-16f * ao * ao;
      }
    }
    const float E = warp_sum_f(errsum) * 1.01f;  // 1.01: the float sums' own rounding (< 2^-18)
    __syncwarp();
    // The cdf scan in exact 64-bit fixed point: F fraction bits with every entry
    // below 2^54 and the total below 2^62 (m <= 256); each entry is off by at most
    // half a unit (2^-54 of the largest entry).
    unsigned long long pb = 0;
    for (int o = lane; o < m; o += 32) {
      const unsigned long long b = (unsigned long long)__double_as_longlong(pmf[o]);
      pb = b > pb ? b : pb;
    }
    pb = warp_max_u64(pb);
    if (pb == 0ull || (pb >> 52) >= 0x7ffull) {  // zero total, or an infinite / NaN entry
      if (lane == 0) atomicOr(a.err, 1);
    } else {
      const int F = 53 - ((int)(pb >> 52) - 1023);
      unsigned long long run = 0;
      for (int q = 0; q < K; ++q)
        if (o0 + q < m) run += fixed_of_double(pmf[o0 + q], F);
#pragma unroll
      for (int off = 1; off < 32; off <<= 1) {
        const unsigned long long y = __shfl_up_sync(0xffffffffu, run, off);
        if (lane >= off) run += y;
      }
      const unsigned long long tot = __shfl_sync(0xffffffffu, run, 31);
      unsigned long long C = __shfl_up_sync(0xffffffffu, run, 1);
      if (lane == 0) C = 0;
      // numpy's random_sample is N / 2^53 with an integer N < 2^53, so for an
      // integer C: C <= u * tot  <=>  C <= floor(N * tot / 2^53), exactly.
      const unsigned long long Nu = fixed_of_double(uu, 53);
      const unsigned long long ut = (__umul64hi(Nu, tot) << 11) | ((Nu * tot) >> 53);
      // the window in fixed-point units: E 2^(2 Ec + F), plus the scan's and
      // theboss's roundings ((m + 4) 2^-52 of the total, over-counted 4x) and the
      // entries' half units
      const float wf = scale_pow2f(E, 2 * Ec + F);
      unsigned long long W = (wf < 4.0e18f) ? (unsigned long long)wf + 1ull : (1ull << 62);
      W += ((tot >> 50) + 1ull) * (unsigned long long)(m + 4) + (unsigned long long)m;
      int cnt = 0;
      for (int q = 0; q < K; ++q) {
        const int o = o0 + q;
        if (o >= m) break;
        C += fixed_of_double(pmf[o], F);  // the cdf step after output o, times total
        const unsigned long long dlt = C > ut ? C - ut : ut - C;
        near |= (o < m - 1) && dlt <= W;
        cnt += (C <= ut) ? 1 : 0;
      }
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, off);
      idx = cnt < m ? cnt : m - 1;
    }
  } else {
    // ---- float pairs on the FP32 pipe (opt-in) ----
    if (a.k > 1 && a.cur_ff && lane < nd) {  // a scale beyond the float range: apply it in FP64
      const SweepProblem& P = a.probs_cur[j];
      const int sc_exp = (int)((__double_as_longlong(P.scale) >> 52) & 0x7FF) - 1023;
      if (!(sc_exp >= -126 && sc_exp <= 127)) {
        const float4 u = subf_s[w][lane];
        float4 f;
        double_to_ff(ff_to_double(u.x, u.y) * P.scale, f.x, f.y);
        double_to_ff(ff_to_double(u.z, u.w) * P.scale, f.z, f.w);
        subf_s[w][lane] = f;
      }
    }
    if (a.k > 1 && !a.cur_ff && lane < nd) {  // FP64 minors to float pairs
      const double2 v = sub_s[w][lane];
      float4 f;
      double_to_ff(v.x, f.x, f.y);
      double_to_ff(v.y, f.z, f.w);
      subf_s[w][lane] = f;
    }
    __syncwarp();
    // the bound's scale: 2^-Ec, 2^Ec <= max_d |c_d|_1 < 2^(Ec + 1)
    float c1 = 0.0f;
    if (lane < nd) {
      const float4 c = subf_s[w][lane];
      c1 = fabsf(c.x) + fabsf(c.z);
    }
    unsigned cbits = __float_as_uint(c1);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) cbits = max(cbits, __shfl_xor_sync(0xffffffffu, cbits, off));
    const int Ec = (int)(cbits >> 23) - 127;
    if (lane < nd) cn_s[w][lane] = scale_pow2f(c1, -Ec) * 1.0000002f;  // in [0, 2); the lo parts
    __syncwarp();
    const float eps2 = 2.0f * kMinorsErrFF;
    const float gam = 9.094947e-13f;  // 2^-40: the compensated dot products
    float errsum = 0.0f;
    // The dot products run as compensated float-pair sums, |.|^2 as a float pair
    // (stored in the warp's pmf row, float2 per output).
    const float4* UT = a.Uff + (size_t)j * a.mstride;
    const float* UA = a.Uabs + (size_t)j * a.mstride;
    float2* pf = reinterpret_cast<float2*>(pmf_s[w]);
    for (int o = lane; o < full; o += 32) {
      float sr = 0.0f, cr = 0.0f, si = 0.0f, ci = 0.0f, ao = 0.0f, bo = 0.0f;
#pragma unroll 4  // independent gathers in flight
      for (int d = 0; d < nd; ++d) {
        const float4 c = subf_s[w][d];
        const int e = dm_s[w][d] * m + o;
        const float4 u = UT[e];
        const float ua = UA[e];
        ff_dot_acc(sr, cr, 1.0f, c.x, c.y, u.x, u.y);
        ff_dot_acc(sr, cr, -1.0f, c.z, c.w, u.z, u.w);
        ff_dot_acc(si, ci, 1.0f, c.x, c.y, u.z, u.w);
        ff_dot_acc(si, ci, 1.0f, c.z, c.w, u.x, u.y);
        ao = fmaf(cn_s[w][d], ua, ao);
        bo += ua;
      }
      pf[o] = ff_abs2(sr, cr, si, ci);
      const float eo = eps2 * bo + gam * ao;
      errsum += eo * (2.0f * ao + eo);
    }
    if (m > full) {
      const int r = m - full;
      int s = 1;  // lanes per remaining output (a power of two, r * s <= 32)
      while (r * (s << 1) <= 32) s <<= 1;
      const int oi = lane / s, c0 = lane & (s - 1);
      float sr = 0.0f, cr = 0.0f, si = 0.0f, ci = 0.0f, ao = 0.0f, bo = 0.0f;
      if (oi < r) {
#pragma unroll 4  // independent gathers in flight
        for (int d = c0; d < nd; d += s) {
          const float4 c = subf_s[w][d];
          const int e = dm_s[w][d] * m + full + oi;
          const float4 u = UT[e];
          const float ua = UA[e];
          ff_dot_acc(sr, cr, 1.0f, c.x, c.y, u.x, u.y);
          ff_dot_acc(sr, cr, -1.0f, c.z, c.w, u.z, u.w);
          ff_dot_acc(si, ci, 1.0f, c.x, c.y, u.z, u.w);
          ff_dot_acc(si, ci, 1.0f, c.z, c.w, u.x, u.y);
          ao = fmaf(cn_s[w][d], ua, ao);
          bo += ua;
        }
      }
      for (int off = s >> 1; off > 0; off >>= 1) {  // fixed butterfly order over the output's lanes
        const float osr = __shfl_xor_sync(0xffffffffu, sr, off), ocr = __shfl_xor_sync(0xffffffffu, cr, off);
        const float osi = __shfl_xor_sync(0xffffffffu, si, off), oci = __shfl_xor_sync(0xffffffffu, ci, off);
        ff_acc(sr, cr, 1.0f, osr, ocr);
        ff_acc(si, ci, 1.0f, osi, oci);
        ao += __shfl_xor_sync(0xffffffffu, ao, off);
        bo += __shfl_xor_sync(0xffffffffu, bo, off);
      }
      if (oi < r && c0 == 0) {
        pf[full + oi] = ff_abs2(sr, cr, si, ci);
        const float eo = eps2 * bo + gam * ao;
        errsum += eo * (2.0f * ao + eo);
      }
    }
    const float E = warp_sum_f(errsum) * 1.01f;
    __syncwarp();
    float ih = 0.0f, il = 0.0f;
    for (int q = 0; q < K; ++q)
      if (o0 + q < m) ff_acc(ih, il, 1.0f, pf[o0 + q].x, pf[o0 + q].y);
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const float yh = __shfl_up_sync(0xffffffffu, ih, off), yl = __shfl_up_sync(0xffffffffu, il, off);
      if (lane >= off) ff_acc(ih, il, 1.0f, yh, yl);
    }
    const float th = __shfl_sync(0xffffffffu, ih, 31), tl = __shfl_sync(0xffffffffu, il, 31);
    float ch = __shfl_up_sync(0xffffffffu, ih, 1), cl = __shfl_up_sync(0xffffffffu, il, 1);
    if (lane == 0) ch = cl = 0.0f;
    if (!(th > 0.0f && th <= 3.4e38f)) {  // not a positive finite total
      if (lane == 0) atomicOr(a.err, 1);
    } else {
      float uth, utl;
      double_to_ff(uu, uth, utl);
      ff_mul(uth, utl, th, tl);  // u * total
      // the window, scaled by 2^-2Ec: E plus the float-pair scan's error (m + 4) 2^-44 of the total
      const float win = E + (float)(m + 4) * 5.684342e-14f * scale_pow2f(th, -2 * Ec);
      int cnt = 0;
      for (int q = 0; q < K; ++q) {
        if (o0 + q >= m) break;
        ff_acc(ch, cl, 1.0f, pf[o0 + q].x, pf[o0 + q].y);  // ~ cdf * total
        float dh = ch, dl = cl;
        ff_acc(dh, dl, -1.0f, uth, utl);  // normalised: its sign is dh's
        near |= (o0 + q < m - 1) && scale_pow2f(fabsf(dh), -2 * Ec) <= win;
        cnt += (dh <= 0.0f) ? 1 : 0;
      }
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, off);
      idx = cnt < m ? cnt : m - 1;
      if (__any_sync(0xffffffffu, near)) {
        for (int o = lane; o < m; o += 32) {  // the pmf as doubles, in place (same 8-byte slots)
          const float2 v = pf[o];
          pmf_s[w][o] = ff_to_double(v.x, v.y);
        }
      }
    }
  }
  if (__any_sync(0xffffffffu, near)) {
    // theboss's exact sequential evaluation in FP64 on the pmf: Python's sum, the
    // division, numpy's cumsum, the division by the last entry, searchsorted
    __syncwarp();
    double total = 0.0;
    if (lane == 0)
      for (int o = 0; o < m; ++o) total += pmf_s[w][o];
    total = __shfl_sync(0xffffffffu, total, 0);
    for (int o = lane; o < m; o += 32) pmf_s[w][o] = pmf_s[w][o] / total;
    __syncwarp();
    if (lane == 0) {
      double acc = 0.0;
      for (int o = 0; o < m; ++o) {
        acc += pmf_s[w][o];
        pmf_s[w][o] = acc;
      }
      atomicAdd(a.err + 1, 1);
    }
    __syncwarp();
    const double last = pmf_s[w][m - 1];
    int cnt2 = 0;
    for (int o = lane; o < m; o += 32) cnt2 += (pmf_s[w][o] / last <= uu) ? 1 : 0;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) cnt2 += __shfl_xor_sync(0xffffffffu, cnt2, off);
    idx = cnt2 < m ? cnt2 : m - 1;
  }
  if (lane == 0) {
    const uint8_t tv = (uint8_t)(trow_s[w][idx] + 1);
    trow_s[w][idx] = tv;
    T[idx] = tv;
  }
  __syncwarp();
  if (j >= a.A_next) return;

  // ---- the all-minors sweep of level k + 1 ----
  {
    const int mode = __shfl_sync(0xffffffffu, pmv, pop_particle_warp(remw, __shfl_sync(0xffffffffu, idxv, a.k), lane));
    if (lane == 0) {
      const uint8_t sv = (uint8_t)(srow_s[w][mode] + 1);
      srow_s[w][mode] = sv;
      S[mode] = sv;
    }
    if (lane < 8) a.rem[(size_t)j * 8 + lane] = remw;
  }
  __syncwarp();
  int nb = 0, nmul = 0, nf = 0;
  for (int base = 0; base < m; base += 32) {
    const int mode = base + lane;
    const int sv = (mode < m) ? srow_s[w][mode] : 0;
    const unsigned b1 = __ballot_sync(0xffffffffu, sv == 1);
    if (sv == 1) {
      const int pos = nb + __popc(b1 & ((1u << lane) - 1u));
      dm_s[w][pos] = (uint8_t)mode;
      mult_s[w][pos] = 1;
    }
    nb += __popc(b1);
  }
  for (int base = 0; base < m; base += 32) {
    const int mode = base + lane;
    const int sv = (mode < m) ? srow_s[w][mode] : 0;
    const unsigned bm = __ballot_sync(0xffffffffu, sv > 1);
    if (sv > 1) {
      const int pos = nb + nmul + __popc(bm & ((1u << lane) - 1u));
      dm_s[w][pos] = (uint8_t)mode;
      mult_s[w][pos] = (uint8_t)sv;
    }
    nmul += __popc(bm);
  }
  // factors: every output particle (a mode occupied p times gives p factors)
  for (int base = 0; base < m; base += 32) {
    const int mode = base + lane;
    const int tv = (mode < m) ? trow_s[w][mode] : 0;
    int incl = tv;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, incl, off);
      if (lane >= off) incl += y;
    }
    for (int q = 0; q < tv; ++q) fm_s[w][nf + incl - tv + q] = (uint8_t)mode;
    nf += __shfl_sync(0xffffffffu, incl, 31);
  }
  __syncwarp();
  nd = nb + nmul;
  // Glynn form: hold the last binary digit at r = 0 (halving); it moves to the
  // end of the digit list, where its minor row is.
  const int held = (nb > 0) ? 1 : 0;
  if (held) {
    const int src = (lane + 1 < nd) ? lane + 1 : nb - 1;  // rotate entries nb-1 .. nd-1 left by one
    uint8_t dmv = 0, muv = 0;
    if (lane >= nb - 1 && lane < nd) {
      dmv = dm_s[w][src];
      muv = mult_s[w][src];
    }
    __syncwarp();
    if (lane >= nb - 1 && lane < nd) {
      dm_s[w][lane] = dmv;
      mult_s[w][lane] = muv;
    }
    __syncwarp();
  }
  const int nds = nd - held;  // digits of the sweep
  LevelSample ls;
  if (a.next_tab) {
    ls = a.next_tab[j];
  } else {  // every sample of the next level has the same code count and layout
    ls.n_codes = a.next_uni.n_codes;
    ls.n_threads = a.next_uni.n_threads;
    ls.thread_begin = (int64_t)j * a.next_uni.n_threads;
    ls.part_off = (int64_t)j * a.next_uni.part_off;
    ls.pool_off = (int64_t)j * a.next_uni.pool_off;
  }
  // rows: -2 U[out][in] for the sweep's digits; base sums: sum_i S_i U[out][i]
  // over every input mode (all signs +1 at r = 0), exact in fixed point
  longlong2* D = a.pool_next + ls.pool_off;
  #pragma unroll 8  // independent gathers in flight
  for (int e = lane; e < nds * nf; e += 32) {
    const int d = e / nf, f = e - d * nf;
    const longlong2 u = Ufxs[(size_t)fm_s[w][f] * m + dm_s[w][d]];
    D[e] = make_longlong2(-2 * u.x, -2 * u.y);
  }
  longlong2* B = D + (size_t)nds * nf;
  // Float-pair sweeps: factor f is scaled by 2^-(p_f + 1), 2^p_f <= its bound
  // max(sum_d mult_d |Re U|, sum_d mult_d |Im U|) < 2^(p_f + 1) (fixed-point units),
  // so |s_f| < 1 in that scale; fx_to_ff takes the bias 189 - p_f.
  float4* DF = reinterpret_cast<float4*>(B + nf);
  int* fbias = reinterpret_cast<int*>(DF + (size_t)(nb - held) * nf);
  int esum = 0;  // sum_f (p_f + 1)
  for (int f = lane; f < nf; f += 32) {
    long long bx = 0, by = 0;
    unsigned long long ax = 0, ay = 0;
    #pragma unroll 8  // independent gathers in flight
    for (int d = 0; d < nd; ++d) {
      const longlong2 u = Ufxs[(size_t)fm_s[w][f] * m + dm_s[w][d]];
      bx += (long long)mult_s[w][d] * u.x;
      by += (long long)mult_s[w][d] * u.y;
      ax += (unsigned long long)mult_s[w][d] * (unsigned long long)(u.x < 0 ? -u.x : u.x);
      ay += (unsigned long long)mult_s[w][d] * (unsigned long long)(u.y < 0 ? -u.y : u.y);
    }
    B[f] = make_longlong2(bx, by);
    if (a.next_ff) {
      const unsigned long long bnd = ax > ay ? ax : ay;
      const int p = bnd ? 63 - __clzll((long long)bnd) : 0;
      fbias[f] = 189 - p;
      esum += p + 1;
    }
  }
  if (a.next_ff) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) esum += __shfl_xor_sync(0xffffffffu, esum, off);
    __syncwarp();  // fbias written by the other lanes
    #pragma unroll 8  // independent gathers in flight
    for (int e = lane; e < (nb - held) * nf; e += 32) {
      const int d = e / nf, f = e - d * nf;
      const longlong2 u = Ufxs[(size_t)fm_s[w][f] * m + dm_s[w][d]];
      float4 v;
      fx_to_ff(-2 * u.x, fbias[f], v.x, v.y);
      fx_to_ff(-2 * u.y, fbias[f], v.z, v.w);
      DF[e] = v;
    }
  }
  SweepProblem& P = a.probs_next[j];
  P.mult[lane] = (lane < nd) ? mult_s[w][lane] : 0;
  P.mult[lane + 32] = 0;
  a.dmode_next[(size_t)j * 32 + lane] = (lane < nd) ? dm_s[w][lane] : 0;
  if (lane == 0) {
    // S_i minor_i = 2^-(k-1) (halved) or 2^-k (not) times the Glynn sum, k = nf + 1
    // input particles; the kernel accumulates half of it.
    P.nd = nds;
    P.nb = nb - held;
    P.nf = nf;
    P.kind = kGlynn;
    P.parity0 = 0;
    P.fx = a.fx;
    P.has_base = 1;
    P.out_idx = j;
    P.n_codes = ls.n_codes;
    P.thread_begin = ls.thread_begin;
    P.n_threads = ls.n_threads;
    P.mat_off = ls.pool_off;
    P.base_off = ls.pool_off + (int64_t)nds * nf;
    P.part_off = ls.part_off;
    // float pairs: the factors' scales 2^(p_f + 1 - fx) multiply the product
    P.ff_off = a.next_ff ? ls.pool_off + (int64_t)(nds + 1) * nf : 0;
    const int e2 = (held ? -(nf - 1) : -nf) + (a.next_ff ? esum - nf * a.fx : 0);
    P.scale = (e2 >= -1022 && e2 <= 1023) ? __longlong_as_double((long long)(e2 + 1023) << 52) : ldexp(1.0, e2);
    P.fixed_digit = held;
    P.group = a.next_tab ? 1 : a.next_group;
  }
}

// ---------------------------------------------------------------------------
// Host orchestration: prepare (schedule, upload, capture) / launch / collect.
// ---------------------------------------------------------------------------
struct GccbRun {
  int N = 0, m = 0, n = 0, Lmax = 0;
  int slot = 0;  // which set of device buffers, pinned buffer and graph
  std::vector<int> order;
  size_t h2d_bytes = 0, d2h_bytes = 0;
  uint8_t* dT = nullptr;
  int* derr = nullptr;
  int kernels = 0, sweeps = 0;
  double sweep_flops = 0.0;  // flops of all sweep launches (the Glynn form's codes)
  double ref_flops = 0.0;    // the same count over theboss's Ryser-form codes
  double ff_inst = 0.0;      // FP32 instructions of the float-pair sweeps (model count per code)
  bool f64 = true;           // FP64 sweeps and pmf (false: float pairs)
  std::vector<cudaEvent_t> ev;  // 2 per sweep level when timing
};
// Draws decided by the exact sequential rule (a cdf step within the error window
// of the uniform), summed over the sampler's calls until read (boss_gccb_near_ties).
static int64_t g_gccb_near_ties = 0;
// Independent slots (device buffers cx->gccb[8 slot .. 8 slot + 7], a pinned
// staging buffer, a graph and a stream each): the host can plan one batch while
// the GPU runs the others, and their kernels overlap on the GPU.
constexpr int kGccbSlots = 4;
constexpr int kGccbPipelineMin = 4096;  // samples from which a call runs as pipelined parts
constexpr int kGccbMaxParts = 8;         // parts of a pipelined call at most
static cudaGraphExec_t g_gccb_exec[kGccbSlots] = {};
static void* g_gccb_pinned[kGccbSlots] = {};
static size_t g_gccb_pinned_bytes[kGccbSlots] = {};

static int ensure_slot_pinned(int slot, size_t bytes) {
  if (g_gccb_pinned_bytes[slot] >= bytes) return kOk;
  if (g_gccb_pinned[slot]) cudaFreeHost(g_gccb_pinned[slot]);
  g_gccb_pinned[slot] = nullptr;
  g_gccb_pinned_bytes[slot] = 0;
  const size_t cap = std::max(bytes, (size_t)1 << 20);
  cudaError_t e = cudaHostAlloc(&g_gccb_pinned[slot], cap, cudaHostAllocDefault);
  if (e != cudaSuccess) return fail_cuda(e, "pinned sampler buffer");
  g_gccb_pinned_bytes[slot] = cap;
  return kOk;
}

static void destroy_events(GccbRun& R) {
  for (auto e : R.ev) cudaEventDestroy(e);
  R.ev.clear();
}

// The Laplace step's coalesced layouts, out[mat][i][o] from U[mat][o][i]: as
// 27-bit limbs of U * 2^lfx rounded (FP64 pmf) or as float pairs, and |Re| + |Im|
// in float (the pmf error bound).
__global__ void transpose_matrices_kernel(const double2* __restrict__ U, void* __restrict__ out,
                                          float* __restrict__ uabs, int m, int64_t count, int f64, int lfx) {
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= count) return;
  const int64_t mm = (int64_t)m * m;
  const int64_t mat = idx / mm, r = idx - mat * mm;
  const int o = (int)(r / m), i = (int)(r - (int64_t)o * m);
  const double2 v = U[idx];
  const int64_t t = mat * mm + (int64_t)i * m + o;
  if (f64) {
    const long long X = __double2ll_rn(ldexp(v.x, lfx)), Y = __double2ll_rn(ldexp(v.y, lfx));  // |.| < 2^53
    reinterpret_cast<int4*>(out)[t] =
        make_int4((int)(X & 0x7FFFFFF), (int)(X >> 27), (int)(Y & 0x7FFFFFF), (int)(Y >> 27));
  } else {
    float4 f;
    double_to_ff(v.x, f.x, f.y);
    double_to_ff(v.y, f.z, f.w);
    reinterpret_cast<float4*>(out)[t] = f;
  }
  uabs[t] = __double2float_ru(fabs(v.x) + fabs(v.y));  // rounded up: an upper bound
}

__global__ void to_fixed_kernel(const double* __restrict__ x, long long* __restrict__ y, int64_t count, int fx) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) y[i] = __double2ll_rn(ldexp(x[i], fx));  // exact scaling, round to nearest even
}

// ---------------------------------------------------------------------------
// Autotuned launch shapes.  Per level the planner picks a split (threads per
// sample, from the level's code count and the resident threads of the kernel)
// and the size G of the thread groups that sum their minors inside the sweep.
// boss_gccb_autotune times candidate shapes on the caller's workload and keeps,
// per (arithmetic, level, sample-count bucket), the split's power-of-two shift
// and G's cap that ran fastest; the winners are cached in-process and on disk,
// keyed by the GPU's name.
// ---------------------------------------------------------------------------
struct LevelTune {
  int shift = 0;  // threads per sample = heuristic * 2^shift (clamped to [1, codes])
  int gmax = 0;   // cap of the group size G (0: the heuristic's)
};
static std::map<uint64_t, LevelTune> g_level_tune;
static bool g_tune_loaded = false;
static std::string g_tune_gpu;
static int g_pipeline_shift = 4;   // the pipelined first part is count >> shift (tuned: 1..6)
static int g_pipeline_growth = 2;  // each later part is this many times the one before (tuned: 1..4)
static const LevelTune* g_tune_force = nullptr;  // while tuning: one shape for every level
static std::vector<LevelTune> g_tune_force_level;  // while tuning: a shape per level (index k)

static inline int sample_bucket(int64_t A) {
  int b = 0;
  while ((A >> (b + 1)) > 0 && b < 40) ++b;
  return b;  // floor(log2(A))
}
static inline uint64_t tune_key(bool f64, int k, int64_t A) {
  return ((uint64_t)(f64 ? 1 : 0) << 32) | ((uint64_t)k << 16) | (uint64_t)sample_bucket(A);
}
static std::string tune_path() {
  const char* p = getenv("BOSS_TUNE_CACHE");
  if (p && *p) return p;
  const char* h = getenv("HOME");
  return std::string(h && *h ? h : "/tmp") + "/.cache/theboss_gb300/gccb_tune.txt";
}
// The cache file: one line per entry, "<gpu name>|<key>|<shift>|<gmax>", and
// "<gpu name>|pipeline|<shift>|<parts>".  Lines of other GPUs are kept as they are.
static void tune_load(int device) {
  if (g_tune_loaded) return;
  g_tune_loaded = true;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) {
    cudaGetLastError();
    return;
  }
  g_tune_gpu = prop.name;
  FILE* f = fopen(tune_path().c_str(), "r");
  if (!f) return;
  char line[512];
  while (fgets(line, sizeof(line), f)) {
    std::string l(line);
    const size_t a = l.find('|');
    if (a == std::string::npos || l.substr(0, a) != g_tune_gpu) continue;
    const std::string rest = l.substr(a + 1);
    unsigned long long key = 0;
    int x = 0, y = 0;
    if (sscanf(rest.c_str(), "pipeline|%d|%d", &x, &y) >= 1) {
      if (x >= 1 && x <= 6) g_pipeline_shift = x;
      if (y >= 1 && y <= 4) g_pipeline_growth = y;
    } else if (sscanf(rest.c_str(), "%llu|%d|%d", &key, &x, &y) == 3) {
      g_level_tune[(uint64_t)key] = LevelTune{std::max(-3, std::min(x, 3)), std::max(0, std::min(y, 128))};
    }
  }
  fclose(f);
}
static void tune_save() {
  const std::string path = tune_path();
  std::vector<std::string> keep;
  if (FILE* f = fopen(path.c_str(), "r")) {
    char line[512];
    while (fgets(line, sizeof(line), f)) {
      std::string l(line);
      if (l.compare(0, g_tune_gpu.size() + 1, g_tune_gpu + "|") != 0) keep.push_back(l);
    }
    fclose(f);
  }
  for (size_t i = path.find('/', 1); i != std::string::npos; i = path.find('/', i + 1))
    mkdir(path.substr(0, i).c_str(), 0755);  // best effort: an unwritable cache only loses the cache
  FILE* f = fopen(path.c_str(), "w");
  if (!f) return;
  for (const std::string& l : keep) fputs(l.c_str(), f);
  for (const auto& kv : g_level_tune)
    fprintf(f, "%s|%llu|%d|%d\n", g_tune_gpu.c_str(), (unsigned long long)kv.first, kv.second.shift, kv.second.gmax);
  fprintf(f, "%s|pipeline|%d|%d\n", g_tune_gpu.c_str(), g_pipeline_shift, g_pipeline_growth);
  fclose(f);
}
static LevelTune level_tune(bool f64, int k, int64_t A) {
  if (g_tune_force) return *g_tune_force;
  if (k < (int)g_tune_force_level.size()) return g_tune_force_level[k];
  const auto it = g_level_tune.find(tune_key(f64, k, A));
  return it == g_level_tune.end() ? LevelTune{} : it->second;
}

// Slot 0 runs on the library's stream, slots 1.. on the context's sampler
// streams, so that the parts of a pipelined call overlap on the GPU (one part's
// latency-bound first levels beside another's heavy ones).
static inline cudaStream_t slot_stream(Context* cx, int slot) { return slot ? cx->sampler_streams[slot - 1] : cx->stream; }

// matrices: n_mats complex m x m matrices, U[out][in]; one for every sample
// (n_mats == 1) or one per sample (n_mats == number of samples).
// timing: 0 none; 1 an event pair around every sweep launch; 2 an event pair
// around every level (its sweep and its finalize).
static int gccb_prepare(Context* cx, const double* matrix, int n_mats, int m, Draws& D, int timing, GccbRun& R,
                        int slot = 0) {
  const int N = (int)D.L.size();
  tune_load(cx->device);  // the tuned shapes of an earlier process, if any (once per process)
  R.slot = slot;
  DeviceBuffer* B = cx->gccb + 8 * slot;
  const int n = std::max(D.n, 1);
  const std::vector<int32_t>& L = D.L;
  // Single-occupied inputs: every sample at level k sweeps 2^(k-1) Glynn-form codes
  // over k digits, whichever particles it popped.  Binned inputs need the popped
  // modes to plan.
  if (D.binned && D.modes.empty()) modes_from_draws(D);
  R.N = N;
  R.m = m;
  R.n = n;
  // samples by particle count, descending, stable (a counting sort: L <= 255)
  int Lmax = 0;
  std::vector<int> cnt(257, 0);
  for (int s = 0; s < N; ++s) {
    cnt[L[s]]++;
    Lmax = std::max(Lmax, (int)L[s]);
  }
  std::vector<int> A(Lmax + 2, 0);  // samples with at least k particles
  for (int k = Lmax; k >= 1; --k) A[k] = A[k + 1] + cnt[k];
  {
    std::vector<int> pos(Lmax + 2, 0);
    for (int l = Lmax, p = 0; l >= 0; --l) {
      pos[l] = p;
      p += cnt[l];
    }
    R.order.resize(N);
    for (int s = 0; s < N; ++s) R.order[pos[L[s]]++] = s;
  }
  const std::vector<int>& order = R.order;
  R.Lmax = Lmax;
  // fixed point: |row sum| <= n * max |component of U|
  double umax = 0.0;
  for (size_t i = 0; i < (size_t)2 * m * m * n_mats; ++i) umax = std::max(umax, std::fabs(matrix[i]));
  int ex = 0;
  std::frexp(std::max(umax, 1e-300) * std::max(n, 1), &ex);
  const int fx = std::max(-900, std::min(61 - ex, 200));
  // the Laplace step's fixed point: |U| * 2^lfx < 2^53 (umax < 2^eu)
  int eu = 0;
  std::frexp(std::max(umax, 1e-300), &eu);
  const int lfx = std::max(-900, std::min(53 - eu, 1000));
  // Per-level layout (levels 2..Lmax need sweeps).
  std::vector<std::vector<LevelSample>> tab(Lmax + 2);
  std::vector<int64_t> lvl_threads(Lmax + 2, 0), lvl_parts(Lmax + 2, 0), lvl_pool(Lmax + 2, 0);
  // Code count and digit count of every (level, active sample), walked
  // incrementally per sample: adding a particle to mode a multiplies the code
  // count by (occ_a + 2) / (occ_a + 1).
  std::vector<std::vector<uint64_t>> lvl_codes(Lmax + 2);
  std::vector<std::vector<int>> lvl_nd(Lmax + 2);
  std::vector<char> ffl(Lmax + 2, 0);  // level k's sweep runs on float pairs
  // FP64 (the default): FP64 sweeps and an FP64 pmf; float pairs where the
  // float-pair sweep exists for the level's factor count, and a float-pair pmf
  const bool f64 = (g_minors_arith != 0);
  R.f64 = f64;
  for (int k = 2; k <= Lmax; ++k) ffl[k] = (!f64 && minors_ff_available(k - 1)) ? 1 : 0;
  // FP32 instructions per code of a float-pair sweep with nf = k - 1 factors
  auto ff_per_code = [&](int k) { return ffl[k] ? 47.5625 * (k - 1) : 0.0; };
  R.sweep_flops = 0.0;
  R.ref_flops = 0.0;
  R.ff_inst = 0.0;
  if (!D.binned) {
    for (int k = 2; k <= Lmax; ++k) {
      R.sweep_flops += (double)A[k] * std::ldexp(9.0 * k - 12.0, k - 1);
      R.ref_flops += (double)A[k] * std::ldexp(9.0 * k - 12.0, k);
      R.ff_inst += (double)A[k] * std::ldexp(ff_per_code(k), k - 1);
    }
  } else {
    for (int k = 2; k <= Lmax; ++k) {
      lvl_codes[k].resize(A[k]);
      lvl_nd[k].resize(A[k]);
    }
    std::vector<uint8_t> occ(m, 0);
    for (int jj = 0; jj < A[1]; ++jj) {
      const int s = order[jj];
      uint64_t c = 1;  // prod (S_i + 1): theboss's Guan codes
      int nd = 0, singles = 0;
      for (int k = 1; k <= L[s]; ++k) {
        const int md = D.modes[(size_t)s * n + (k - 1)];
        c = c / ((uint64_t)occ[md] + 1) * ((uint64_t)occ[md] + 2);
        if (occ[md] == 0) ++nd;
        singles += (occ[md] == 0) ? 1 : (occ[md] == 1 ? -1 : 0);
        occ[md]++;
        if (k >= 2) {
          const uint64_t cg = singles > 0 ? c / 2 : c;  // Glynn form: one single digit held
          lvl_codes[k][jj] = cg;
          lvl_nd[k][jj] = nd;
          // flops per code of the all-minors sweep: (k-1) complex adds, (k-2) complex
          // products, one sign, k/2 real-weighted adds = 9k - 12; theboss's Ryser
          // form sweeps c codes, the Glynn form cg
          R.sweep_flops += (double)cg * (9.0 * k - 12.0);
          R.ff_inst += (double)cg * ff_per_code(k);
          R.ref_flops += (double)c * (9.0 * k - 12.0);
        }
      }
      for (int k = 0; k < L[s]; ++k) occ[D.modes[(size_t)s * n + k]] = 0;
    }
  }
  std::vector<char> uniform(Lmax + 2, 0);
  std::vector<LevelSample> uni_lvl(Lmax + 2);
  std::vector<int> grp(Lmax + 2, 1);
  std::vector<char> red(Lmax + 2, 0);  // level k's partial rows summed by gccb_partials_reduce_kernel
  int64_t max_red = 0;                 // samples of the largest such level
  for (int k = 2; k <= Lmax; ++k) {
    const int Ak = A[k];
    const std::vector<uint64_t>& codes = lvl_codes[k];
    const std::vector<int>& ndv = lvl_nd[k];
    // k input particles: at most k distinct modes, so at most k rows of minors per thread
    const int64_t resident = sweep_resident_minors(k - 1, std::min(k, kMaxMinorDigits), cx->sm_count, ffl[k]);
    // pool per sample: rows of D and the base sums; float pairs add the float-pair
    // rows of the binary digits and the factors' biases
    auto pool_units = [&](int nd_) { return (int64_t)(ffl[k] ? 2 * nd_ + 2 : nd_ + 1) * (k - 1); };
    bool same = true;
    uint64_t code0 = 1ull << (k - 1);
    int nd0 = k;
    if (D.binned) {
      code0 = codes[0];
      nd0 = ndv[0];
      for (int jj = 1; jj < Ak && same; ++jj) same = (codes[jj] == code0 && ndv[jj] == nd0);
    }
    if (same) {  // one small descriptor instead of a per-sample table
      const double total = (double)code0 * Ak;
      const double want = std::max<double>(Ak, std::min<double>((double)resident, total / kMinCodesPerThread));
      int64_t tps = std::max<int64_t>(1, std::min<int64_t>((int64_t)code0, (int64_t)(want / Ak)));
      const LevelTune lt = level_tune(f64, k, Ak);
      if (lt.shift > 0) tps = std::min<int64_t>((int64_t)code0, tps << lt.shift);
      if (lt.shift < 0) tps = std::max<int64_t>(1, tps >> -lt.shift);
      // Each aligned group of G threads of a sample sums its minors inside the sweep:
      // the largest G (up to a block of 128, when the launch's threads then fill
      // whole blocks) that costs at most 2% of the sample's threads.
      int G = 128;
      if (lt.gmax > 0) G = std::min(G, lt.gmax);
      auto ok = [&](int g) {
        if (!(tps >= g && (double)(tps / g * g) >= 0.98 * (double)tps)) return false;
        return g <= 32 || ((tps / g * g) * (int64_t)Ak) % 128 == 0;
      };
      while (G > 1 && !ok(G)) G >>= 1;
      tps = tps / G * G;
      grp[k] = G;
      uniform[k] = 1;
      uni_lvl[k].n_codes = (int64_t)code0;
      uni_lvl[k].thread_begin = 0;
      uni_lvl[k].n_threads = tps;
      uni_lvl[k].part_off = tps * nd0;
      uni_lvl[k].pool_off = pool_units(nd0);
      if (!ffl[k] && tps / G >= kReduceMinParts && Ak <= kReduceMaxSamples && nd0 <= 32) {
        red[k] = 1;
        max_red = std::max<int64_t>(max_red, Ak);
      }
      lvl_threads[k] = tps * Ak;
      lvl_parts[k] = tps * nd0 * Ak;
      lvl_pool[k] = pool_units(nd0) * Ak;
      continue;
    }
    std::vector<int64_t> nthr;
    {
      const LevelTune lt = level_tune(f64, k, Ak);
      const int64_t res = lt.shift >= 0 ? resident << lt.shift : std::max<int64_t>(1, resident >> -lt.shift);
      partition_threads(codes, res, nthr);
    }
    auto& t = tab[k];
    t.resize(Ak);
    int64_t threads = 0, parts = 0, pool = 0;
    for (int jj = 0; jj < Ak; ++jj) {
      LevelSample ls;
      ls.n_codes = (int64_t)codes[jj];
      ls.thread_begin = threads;
      ls.n_threads = nthr[jj];
      ls.part_off = parts;
      ls.pool_off = pool;
      threads += nthr[jj];
      parts += nthr[jj] * ndv[jj];
      pool += pool_units(ndv[jj]);
      t[jj] = ls;
    }
    lvl_threads[k] = threads;
    lvl_parts[k] = parts;
    lvl_pool[k] = pool;
  }
  int64_t max_parts = 1, max_pool = 1;
  for (int k = 2; k <= Lmax; ++k) {
    max_parts = std::max(max_parts, lvl_parts[k]);
    max_pool = std::max(max_pool, lvl_pool[k]);
  }
  // Arena (one H2D copy): err | level tables | randint results | particle modes | uniforms | U | U fixed-point
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  size_t off = 0;
  const size_t o_err = off; off = al(off + 2 * sizeof(int));
  std::vector<size_t> o_tab(Lmax + 2, 0);
  for (int k = 2; k <= Lmax; ++k) { o_tab[k] = off; off = al(off + sizeof(LevelSample) * tab[k].size()); }
  const size_t o_ord = off; off = al(off + sizeof(int32_t) * (size_t)N);
  const size_t o_idx = off; off = al(off + (size_t)N * n);
  const size_t o_pm = off; off = al(off + (size_t)N * n);
  const size_t o_np = off; off = al(off + (size_t)N);
  const size_t o_uni = off; off = al(off + sizeof(double) * (size_t)N * n);
  const size_t o_U = off; off = al(off + sizeof(double2) * (size_t)m * m * n_mats);
  const size_t arena = off;
  R.h2d_bytes = arena;
  R.d2h_bytes = (size_t)N * m + 2 * sizeof(int);
  int st;
  if ((st = ensure(B[0], arena))) return st;
  if ((st = ensure(B[1], (size_t)N * m * 2))) return st;                              // S | T
  if ((st = ensure(B[2], sizeof(SweepProblem) * (size_t)A[1] * 2 + 512))) return st;  // problems x2
  if ((st = ensure(B[3], (size_t)A[1] * 32 * 2))) return st;                          // digit modes x2
  if ((st = ensure(B[4], sizeof(longlong2) * (size_t)max_pool * 2 + 512))) return st;  // rows x2
  if ((st = ensure(B[5], sizeof(double2) * (size_t)(max_parts + 32 * max_red)))) return st;  // partials | sums
  if ((st = ensure(B[6], sizeof(uint32_t) * 8 * (size_t)N))) return st;                // particles left
  // U fixed point | U^T (doubles or float pairs) | U^T 1-norms
  if ((st = ensure(B[7], 36 * (size_t)m * m * n_mats + 256))) return st;
  if ((st = ensure_slot_pinned(slot, std::max(arena, al((size_t)N * m) + 256)))) return st;
  char* h = (char*)g_gccb_pinned[slot];
  memset(h, 0, o_ord);
  for (int k = 2; k <= Lmax; ++k) memcpy(h + o_tab[k], tab[k].data(), sizeof(LevelSample) * tab[k].size());
  // The draws stay in input order (bulk copies); the kernels reach a sample's
  // row through the level-order permutation.
  memcpy(h + o_ord, order.data(), sizeof(int32_t) * (size_t)N);
  memcpy(h + o_idx, D.idx.data(), (size_t)N * n);
  memcpy(h + o_pm, D.particles.data(), (size_t)N * n);
  memcpy(h + o_np, D.nparticles.data(), (size_t)N);
  memcpy(h + o_uni, D.u.data(), sizeof(double) * (size_t)N * n);
  const size_t mm = (size_t)m * m;
  if (n_mats > 1) {  // instances: matrices in level order
    for (int jj = 0; jj < N; ++jj)
      memcpy(h + o_U + sizeof(double2) * mm * jj, matrix + 2 * mm * order[jj], sizeof(double2) * mm);
  } else {
    memcpy(h + o_U, matrix, sizeof(double2) * mm);
  }
  char* d = (char*)B[0].ptr;
  uint8_t* dS = (uint8_t*)B[1].ptr;
  R.dT = dS + (size_t)N * m;
  R.derr = (int*)(d + o_err);
  SweepProblem* probs[2] = {(SweepProblem*)B[2].ptr, (SweepProblem*)B[2].ptr + A[1]};
  uint8_t* dmode[2] = {(uint8_t*)B[3].ptr, (uint8_t*)B[3].ptr + (size_t)A[1] * 32};
  longlong2* pool[2] = {(longlong2*)B[4].ptr, (longlong2*)B[4].ptr + max_pool};
  double2* partials = (double2*)B[5].ptr;
  double2* reduced = partials + max_parts;  // 32 per sample of a level with red[k]
  cudaStream_t s = slot_stream(cx, slot);
  cudaError_t e = cudaMemcpyAsync(d, h, arena, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return fail_cuda(e, "H2D sampler arena");
  longlong2* dUfx = (longlong2*)B[7].ptr;
  void* dUt = (void*)(dUfx + mm * n_mats);  // 16 bytes per entry either way
  float* dUabs = (float*)((char*)dUt + 16 * mm * n_mats);
  {
    const int64_t cnt = (int64_t)2 * mm * n_mats;
    to_fixed_kernel<<<(unsigned)((cnt + 255) / 256), 256, 0, s>>>((const double*)(d + o_U), (long long*)dUfx, cnt, fx);
    if ((e = cudaGetLastError()) != cudaSuccess) return fail_cuda(e, "fixed-point matrices");
    const int64_t cnt2 = (int64_t)mm * n_mats;
    transpose_matrices_kernel<<<(unsigned)((cnt2 + 255) / 256), 256, 0, s>>>((const double2*)(d + o_U), dUt, dUabs,
                                                                              m, cnt2, f64 ? 1 : 0, lfx);
    if ((e = cudaGetLastError()) != cudaSuccess) return fail_cuda(e, "transposed matrices");
  }
  destroy_events(R);
  if (timing) {
    R.ev.resize(2 * (size_t)std::max(timing == 2 ? Lmax : Lmax - 1, 0));
    for (auto& ev : R.ev)
      if ((e = cudaEventCreate(&ev)) != cudaSuccess) return fail_cuda(e, "event create");
  }
  // Capture the level loop into one graph.
  cudaGetLastError();
  cudaGraph_t graph = nullptr;
  e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return fail_cuda(e, "begin capture");
  R.kernels = 0;
  R.sweeps = 0;
  cudaError_t le = cudaMemsetAsync(dS, 0, (size_t)N * m * 2, s);
  for (int k = 1; k <= Lmax && le == cudaSuccess; ++k) {
    const int cur = k & 1, nxt = (k + 1) & 1;
    if (k >= 2) {
      SweepLaunch SL;
      SL.probs = probs[cur];
      SL.n_probs = A[k];
      SL.pool = pool[cur];
      SL.total_threads = lvl_threads[k];
      SL.partials = partials;
      SL.grid = (int)((lvl_threads[k] + 127) / 128);
      SL.rows = std::min(k, kMaxMinorDigits);
      SL.uniform_threads = uniform[k] ? uni_lvl[k].n_threads : 0;
      if (timing == 1) le = cudaEventRecordWithFlags(R.ev[2 * (k - 2)], s, cudaEventRecordExternal);
      if (timing == 2) le = cudaEventRecordWithFlags(R.ev[2 * (k - 1)], s, cudaEventRecordExternal);
      if (le == cudaSuccess) le = launch_sweep(k - 1, ffl[k] ? SweepOp::kMinorsFF : SweepOp::kMinors, SL, s);
      if (timing == 1 && le == cudaSuccess)
        le = cudaEventRecordWithFlags(R.ev[2 * (k - 2) + 1], s, cudaEventRecordExternal);
      if (le != cudaSuccess) break;
      ++R.kernels;
      ++R.sweeps;
      if (red[k]) {
        gccb_partials_reduce_kernel<<<dim3((unsigned)A[k], (unsigned)std::min(k, 32)), 128, 0, s>>>(probs[cur],
                                                                                                 partials, reduced);
        if ((le = cudaGetLastError()) != cudaSuccess) break;
        ++R.kernels;
      }
    }
    FinalizeArgs fa;
    fa.k = k;
    fa.A = A[k];
    fa.A_next = (k < Lmax) ? A[k + 1] : 0;
    fa.m = m;
    fa.n = n;
    fa.fx = fx;
    fa.Ufx = dUfx;
    fa.Uff = f64 ? nullptr : (const float4*)dUt;
    fa.Ulimb = f64 ? (const int4*)dUt : nullptr;
    fa.lfx = lfx;
    fa.Uabs = dUabs;
    fa.mstride = (n_mats > 1) ? (int64_t)mm : 0;
    fa.npart = (const uint8_t*)(d + o_np);
    fa.order = (const int32_t*)(d + o_ord);
    fa.S = dS;
    fa.T = R.dT;
    fa.idx = (const uint8_t*)(d + o_idx);
    fa.pmode = (const uint8_t*)(d + o_pm);
    fa.rem = (uint32_t*)B[6].ptr;
    fa.uni = (const double*)(d + o_uni);
    fa.probs_cur = probs[cur];
    fa.dmode_cur = dmode[cur];
    fa.partials = partials;
    fa.reduced = (k >= 2 && red[k]) ? reduced : nullptr;
    fa.probs_next = probs[nxt];
    fa.dmode_next = dmode[nxt];
    fa.pool_next = pool[nxt];
    fa.next_tab = (k < Lmax && !uniform[k + 1]) ? (const LevelSample*)(d + o_tab[k + 1]) : nullptr;
    fa.next_uni = (k < Lmax) ? uni_lvl[k + 1] : LevelSample{};
    fa.next_group = (k < Lmax) ? grp[k + 1] : 1;
    fa.next_ff = (k < Lmax) ? ffl[k + 1] : 0;
    fa.cur_ff = (k >= 2) ? ffl[k] : 0;
    fa.err = R.derr;
    if (timing == 2 && k == 1) le = cudaEventRecordWithFlags(R.ev[0], s, cudaEventRecordExternal);
    if (le != cudaSuccess) break;
    if (f64)
      gccb_finalize_kernel<true><<<(A[k] + kFinWarps - 1) / kFinWarps, kFinWarps * 32, 0, s>>>(fa);
    else
      gccb_finalize_kernel<false><<<(A[k] + kFinWarps - 1) / kFinWarps, kFinWarps * 32, 0, s>>>(fa);
    le = cudaGetLastError();
    if (timing == 2 && le == cudaSuccess)
      le = cudaEventRecordWithFlags(R.ev[2 * (k - 1) + 1], s, cudaEventRecordExternal);
    ++R.kernels;
  }
  e = cudaStreamEndCapture(s, &graph);
  if (le != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    return fail_cuda(le, "sampler launch during capture");
  }
  if (e != cudaSuccess) return fail_cuda(e, "end capture");
  bool updated = false;
  cudaGraphExec_t& exec = g_gccb_exec[slot];
  if (exec) {
    cudaGraphExecUpdateResultInfo info;
    if (cudaGraphExecUpdate(exec, graph, &info) == cudaSuccess) {
      updated = true;
    } else {
      cudaGetLastError();
      cudaGraphExecDestroy(exec);
      exec = nullptr;
    }
  }
  if (!updated) {
    e = cudaGraphInstantiate(&exec, graph, 0);
    if (e != cudaSuccess) {
      cudaGraphDestroy(graph);
      exec = nullptr;
      return fail_cuda(e, "graph instantiate");
    }
  }
  cudaGraphDestroy(graph);
  return kOk;
}

static int gccb_launch(Context* cx, int slot = 0) {
  cudaError_t e = cudaGraphLaunch(g_gccb_exec[slot], slot_stream(cx, slot));
  return e == cudaSuccess ? kOk : fail_cuda(e, "graph launch");
}

// Queues the copies of a run's samples and status into its slot's pinned buffer.
static int gccb_queue_results(Context* cx, GccbRun& R) {
  cudaStream_t s = slot_stream(cx, R.slot);
  char* h = (char*)g_gccb_pinned[R.slot];
  cudaError_t e = cudaMemcpyAsync(h, R.dT, (size_t)R.N * R.m, cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess) return fail_cuda(e, "D2H samples");
  int* herr = (int*)(h + (((size_t)R.N * R.m + 255) & ~(size_t)255));
  e = cudaMemcpyAsync(herr, R.derr, 2 * sizeof(int), cudaMemcpyDeviceToHost, s);
  return e == cudaSuccess ? kOk : fail_cuda(e, "D2H status");
}

// After the stream is synchronised: the status, then the samples in input order.
static int gccb_read_results(const GccbRun& R, int32_t* samples_out) {
  const char* h = (const char*)g_gccb_pinned[R.slot];
  const int* herr = (const int*)(h + (((size_t)R.N * R.m + 255) & ~(size_t)255));
  g_gccb_near_ties += herr[1];
  if (herr[0]) {
    set_error("probabilities contain NaN (a pmf summed to zero or a non-finite value)");
    return kErrPmf;
  }
  if (samples_out) {
    const uint8_t* hT = (const uint8_t*)h;
    for (int jj = 0; jj < R.N; ++jj) {
      int32_t* row = samples_out + (size_t)R.order[jj] * R.m;
      for (int i = 0; i < R.m; ++i) row[i] = hT[(size_t)jj * R.m + i];
    }
  }
  return kOk;
}

static int gccb_collect(Context* cx, GccbRun& R, int32_t* samples_out) {
  int st = gccb_queue_results(cx, R);
  if (st) return st;
  cudaError_t e = cudaStreamSynchronize(slot_stream(cx, R.slot));
  if (e != cudaSuccess) return fail_cuda(e, "sampler");
  return gccb_read_results(R, samples_out);
}

static int run_gccb(Context* cx, const double* matrix, int n_mats, int m, Draws& D, int32_t* samples_out) {
  if (D.L.empty()) return kOk;
  GccbRun R;
  int st = gccb_prepare(cx, matrix, n_mats, m, D, 0, R);
  if (st) return st;
  if ((st = gccb_launch(cx))) return st;
  return gccb_collect(cx, R, samples_out);
}

// Keeps samples [first, first + count) of a replayed batch.
static void keep_rows(Draws& D, int first, int count) {
  const size_t rs = (size_t)std::max(D.n, 1);
  D.particles.erase(D.particles.begin(), D.particles.begin() + first * rs);
  D.particles.resize(count * rs);
  D.nparticles.erase(D.nparticles.begin(), D.nparticles.begin() + first);
  D.nparticles.resize(count);
  D.L.erase(D.L.begin(), D.L.begin() + first);
  D.L.resize(count);
  D.idx.erase(D.idx.begin(), D.idx.begin() + first * rs);
  D.idx.resize(count * rs);
  D.u.erase(D.u.begin(), D.u.begin() + first * rs);
  D.u.resize(count * rs);
  D.modes.clear();
}

// Samples [first, first + count) of the stream of n_samples samples drawn from
// `mt` (advanced over the whole stream).  The API lock is held by the caller.
static int sample_slice_locked(const double* matrix, int m, const int32_t* input_state,
                               const double* particle_weights, int nw, MT19937& mt, int n_samples, int first,
                               int count, int32_t* samples) {
  // Large batches run as pipelined parts: while the GPU samples the parts it has,
  // the host replays and plans the next.  The first part is count >> g_pipeline_shift
  // (a sixteenth unless tuned), so that the GPU starts early, and every later part
  // is g_pipeline_growth times the one before (the last one takes the rest), so
  // that the host's replay of a part (about 0.1 ms per 10^3 samples) stays ahead
  // of the GPU's work on the parts before it.  Parts take the slots in turn
  // (device buffers, pinned buffer, graph and stream each), so consecutive parts
  // overlap on the GPU, one part's latency-bound first and last levels beside
  // another's heavy ones; a slot is reused once its previous part has finished,
  // and that part's rows are read while the GPU works on the other slots.
  std::vector<int> cut(1, first);
  Context* cx = nullptr;
  int st = kOk;
  if (count >= kGccbPipelineMin) {
    if (!(cx = context(&st))) return st;
    tune_load(cx->device);  // the tuned parts of an earlier process, if any
    int64_t size = std::max(count >> g_pipeline_shift, 1), at = 0;
    while (at + size < count && (int)cut.size() < kGccbMaxParts) {
      at += size;
      cut.push_back(first + (int)at);
      size *= g_pipeline_growth;
    }
    if (cut.size() > 2 && count - at < (at - (cut[cut.size() - 2] - first)) / 2)
      cut.pop_back();  // a short tail joins the part before it
  }
  cut.push_back(first + count);
  const int parts = (int)cut.size() - 1;
  GccbRun R[kGccbSlots];
  int in_flight[kGccbSlots];  // the part each slot is running, or -1
  for (int& f : in_flight) f = -1;
  // Waits for the slot's part and writes its rows (or, after an error, only waits).
  auto retire = [&](int slot, bool read) -> int {
    const int p = in_flight[slot];
    if (p < 0) return kOk;
    in_flight[slot] = -1;
    const cudaError_t e = cudaStreamSynchronize(slot_stream(cx, slot));
    if (e != cudaSuccess) return fail_cuda(e, "sampler");
    return read ? gccb_read_results(R[slot], samples + (size_t)(cut[p] - first) * m) : kOk;
  };
  int done = 0;  // stream samples replayed so far
  for (int p = 0; p < parts && !st; ++p) {
    const int slot = p % kGccbSlots;
    Draws D;  // replayed before waiting for the slot: the host's share of the overlap
    const int upto = (p + 1 == parts) ? n_samples : cut[p + 1];  // the last part replays the stream's tail
    if ((st = predraw(input_state, m, particle_weights, nw, mt, upto - done, D))) break;
    if (D.n > kMaxMinorDigits) {
      set_error("the batched sampler supports at most 32 input particles");
      st = kErrLimit;
      break;
    }
    keep_rows(D, cut[p] - done, cut[p + 1] - cut[p]);
    done = upto;
    if ((st = retire(slot, true))) break;
    if (!std::any_of(D.L.begin(), D.L.end(), [](int32_t l) { return l > 0; })) {  // every row empty
      memset(samples + (size_t)(cut[p] - first) * m, 0, sizeof(int32_t) * (size_t)(cut[p + 1] - cut[p]) * m);
      continue;
    }
    if (!cx && !(cx = context(&st))) break;
    in_flight[slot] = p;  // from here on the slot's stream may hold work of this part
    if ((st = gccb_prepare(cx, matrix, 1, m, D, 0, R[slot], slot))) break;
    if ((st = gccb_launch(cx, slot))) break;
    if ((st = gccb_queue_results(cx, R[slot]))) break;
  }
  // The remaining parts in order of their slots; after an error every slot is
  // still drained, so that no copy into a pinned buffer outlives the call.
  for (int slot = 0; slot < kGccbSlots; ++slot) {
    const int rs = retire(slot, st == kOk);
    if (!st) st = rs;
  }
  return st;
}

// Samples with at least k particles, k = 0..Lmax.
static std::vector<int64_t> level_counts(const Draws& D) {
  int Lmax = 0;
  for (int32_t l : D.L) Lmax = std::max(Lmax, (int)l);
  std::vector<int64_t> A(Lmax + 2, 0);
  for (int32_t l : D.L) A[l]++;
  for (int k = Lmax - 1; k >= 0; --k) A[k] += A[k + 1];
  return A;
}

// Whether every level of this workload (the draws of `count` samples from a copy
// of `mt`) already has a tuned entry.
static bool workload_tuned(const int32_t* input_state, int m, const double* weights, int nw, const MT19937& mt,
                           int count) {
  MT19937 t = mt;
  Draws D;
  if (predraw(input_state, m, weights, nw, t, count, D)) return true;  // errors surface in the call itself
  const std::vector<int64_t> A = level_counts(D);
  const bool f64 = (g_minors_arith != 0);
  for (int k = 2; k + 1 < (int)A.size(); ++k)
    if (A[k] > 0 && !g_level_tune.count(tune_key(f64, k, A[k]))) return false;
  return true;
}

// Per-level times (minimum over reps, after one warm-up run) of the graph with
// the current forced shapes; lvl_ms[k] covers level k's sweep and finalize.
static int tune_levels(Context* cx, const double* matrix, int m, Draws& D, int reps, std::vector<double>& lvl_ms) {
  GccbRun R;
  int st = gccb_prepare(cx, matrix, 1, m, D, 2, R);
  if (st) return st;
  lvl_ms.assign(R.Lmax + 2, 1e30);
  for (int it = 0; it <= reps && !st; ++it) {
    if ((st = gccb_launch(cx))) break;
    const cudaError_t e = cudaStreamSynchronize(cx->stream);
    if (e != cudaSuccess) {
      st = fail_cuda(e, "autotune");
      break;
    }
    for (int k = 1; it > 0 && k <= R.Lmax; ++k) {
      float x = 0.f;
      if (cudaEventElapsedTime(&x, R.ev[2 * (k - 1)], R.ev[2 * (k - 1) + 1]) == cudaSuccess)
        lvl_ms[k] = std::min(lvl_ms[k], (double)x);
      else
        cudaGetLastError();
    }
  }
  destroy_events(R);
  return st;
}

// The plain graph's step time (minimum over reps, after one warm-up run).
static int tune_step(Context* cx, const double* matrix, int m, Draws& D, int reps, double& ms) {
  GccbRun R;
  int st = gccb_prepare(cx, matrix, 1, m, D, 0, R);
  if (st) return st;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  ms = 1e30;
  for (int it = 0; it <= reps && !st; ++it) {
    cudaEventRecord(e0, cx->stream);
    if ((st = gccb_launch(cx))) break;
    cudaEventRecord(e1, cx->stream);
    const cudaError_t e = cudaEventSynchronize(e1);
    if (e != cudaSuccess) {
      st = fail_cuda(e, "autotune");
      break;
    }
    float x = 0.f;
    if (it > 0 && cudaEventElapsedTime(&x, e0, e1) == cudaSuccess) ms = std::min(ms, (double)x);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return st;
}

// The tuner: times the levels under power-of-two shifts of the split, then under
// caps of the group size G, keeps each level's fastest shape if the whole step
// gets faster, then times the pipelined parts on end-to-end calls.
// report[0..7]: step ms with the heuristic shapes and with the tuned ones, levels
// whose shape changed, the pipeline shift, end-to-end ms with the default parts
// (shift 4, growth 2) and with the tuned ones (0 when the call is below the
// pipelining size), the sum over levels of each level's own time (sweep to end of
// finalize, heuristic shapes: the step minus it is the graph's time between
// levels), and the growth of the later parts.
static int gccb_autotune_locked(Context* cx, const double* matrix, int m, const int32_t* input_state,
                                const double* weights, int nw, const MT19937& mt0, int n_samples, int reps,
                                double* report) {
  for (int i = 0; i < 8; ++i) report[i] = 0.0;
  MT19937 mt = mt0;
  Draws D;
  int st = predraw(input_state, m, weights, nw, mt, n_samples, D);
  if (st) return st;
  if (D.n > kMaxMinorDigits || D.n < 1) {
    set_error("the batched sampler needs 1..32 input particles");
    return kErrLimit;
  }
  const std::vector<int64_t> A = level_counts(D);
  const int Lmax = (int)A.size() - 2;
  if (Lmax < 1) return kOk;
  const bool f64 = (g_minors_arith != 0);
  struct ForceGuard {
    ~ForceGuard() {
      g_tune_force = nullptr;
      g_tune_force_level.clear();
    }
  } guard;
  const LevelTune none{};
  std::vector<LevelTune> best(Lmax + 1);
  std::vector<double> best_ms, ms;
  double step0 = 0.0, step1 = 0.0;
  g_tune_force = &none;
  if ((st = tune_step(cx, matrix, m, D, reps, step0))) return st;
  if ((st = tune_levels(cx, matrix, m, D, reps, best_ms))) return st;
  for (int k = 1; k <= Lmax; ++k) report[6] += best_ms[k];  // the levels' own time, gaps excluded
  for (int sh : {-2, -1, 1, 2}) {  // the split
    const LevelTune c{sh, 0};
    g_tune_force = &c;
    if ((st = tune_levels(cx, matrix, m, D, reps, ms))) return st;
    for (int k = 2; k <= Lmax; ++k)
      if (ms[k] < 0.97 * best_ms[k]) {
        best_ms[k] = ms[k];
        best[k] = c;
      }
  }
  g_tune_force = nullptr;
  for (int gm : {1, 4, 8, 16}) {  // the group size's cap, with each level's best split
    g_tune_force_level.assign(Lmax + 1, LevelTune{});
    for (int k = 2; k <= Lmax; ++k) g_tune_force_level[k] = LevelTune{best[k].shift, gm};
    if ((st = tune_levels(cx, matrix, m, D, reps, ms))) return st;
    for (int k = 2; k <= Lmax; ++k)
      if (ms[k] < 0.97 * best_ms[k]) {
        best_ms[k] = ms[k];
        best[k].gmax = gm;
      }
  }
  g_tune_force_level = best;
  if ((st = tune_step(cx, matrix, m, D, reps, step1))) return st;
  g_tune_force_level.clear();
  const bool keep = step1 < step0;
  int changed = 0;
  for (int k = 2; k <= Lmax; ++k) {
    if (A[k] <= 0) continue;
    const LevelTune v = keep ? best[k] : LevelTune{};
    g_level_tune[tune_key(f64, k, A[k])] = v;
    changed += (v.shift != 0 || v.gmax != 0) ? 1 : 0;
  }
  report[0] = step0;
  report[1] = keep ? step1 : step0;
  report[2] = changed;
  // The pipelined parts, on end-to-end calls of the same stream: the first part's
  // shift and the growth of the later parts, the default (4, 2) first as the reference.
  report[3] = g_pipeline_shift;
  report[7] = g_pipeline_growth;
  if (n_samples >= kGccbPipelineMin) {
    std::vector<int32_t> out((size_t)n_samples * m);
    double best_e2e = 1e30;
    int best_shift = 4, best_growth = 2;
    std::vector<std::pair<int, int>> cand(1, std::make_pair(4, 2));
    for (int sh = 2; sh <= 6; ++sh)
      for (int gr = 1; gr <= 3; ++gr)
        if (sh != 4 || gr != 2) cand.push_back(std::make_pair(sh, gr));
    for (size_t c = 0; c < cand.size() && !st; ++c) {
      g_pipeline_shift = cand[c].first;
      g_pipeline_growth = cand[c].second;
      double t_min = 1e30;
      for (int it = 0; it <= reps; ++it) {
        MT19937 t = mt0;
        const auto t0 = std::chrono::steady_clock::now();
        if ((st = sample_slice_locked(matrix, m, input_state, weights, nw, t, n_samples, 0, n_samples, out.data())))
          break;
        const double dt = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        if (it > 0) t_min = std::min(t_min, dt);
      }
      if (st) break;
      if (c == 0) report[4] = t_min;
      if (c == 0 || t_min < 0.97 * best_e2e) {
        best_e2e = t_min;
        best_shift = cand[c].first;
        best_growth = cand[c].second;
      }
    }
    g_pipeline_shift = best_shift;
    g_pipeline_growth = best_growth;
    report[3] = best_shift;
    report[7] = best_growth;
    report[5] = best_e2e;
    if (st) return st;
  }
  tune_save();
  return kOk;
}

}  // namespace boss

using namespace boss;

static int load_mt(MT19937& mt, const uint32_t* key, const int32_t* pos) {
  if (!key || !pos || *pos < 0 || *pos > 624) {
    set_error("invalid MT19937 state");
    return kErrArg;
  }
  memcpy(mt.key, key, sizeof(mt.key));
  mt.pos = *pos;
  if (mt.pos < 624) mt.temper_all();
  return kOk;
}

extern "C" {

int boss_gccb_predraw(const int32_t* input_state, int32_t m, const double* particle_weights, int32_t n_weights,
                      uint32_t* mt_key, int32_t* mt_pos, int32_t n_samples, int32_t* particles_kept,
                      int32_t* popped_modes, double* uniforms) {
  if (!input_state || m <= 0 || n_samples < 0 || !particles_kept) {
    set_error("null pointer or bad size");
    return kErrArg;
  }
  MT19937 mt;
  int st = load_mt(mt, mt_key, mt_pos);
  if (st) return st;
  Draws D;
  st = predraw(input_state, m, particle_weights, particle_weights ? n_weights : 0, mt, n_samples, D);
  if (st) return st;
  const std::vector<int32_t>& L = D.L;
  const int n = D.n;
  if (popped_modes) modes_from_draws(D);
  for (int s = 0; s < n_samples; ++s) {
    particles_kept[s] = L[s];
    for (int k = 0; k < n; ++k) {
      if (popped_modes) popped_modes[(size_t)s * n + k] = (k < L[s]) ? D.modes[(size_t)s * n + k] : -1;
      if (uniforms) uniforms[(size_t)s * n + k] = (k < L[s]) ? D.u[(size_t)s * n + k] : 0.0;
    }
  }
  memcpy(mt_key, mt.key, sizeof(mt.key));
  *mt_pos = mt.pos;
  return kOk;
}

int boss_gccb_sample(const double* matrix, int32_t m, const int32_t* input_state, const double* particle_weights,
                     int32_t n_weights, uint32_t* mt_key, int32_t* mt_pos, int32_t n_samples, int32_t* samples) {
  return boss_gccb_sample_slice(matrix, m, input_state, particle_weights, n_weights, mt_key, mt_pos, n_samples, 0,
                                n_samples, samples);
}

int boss_gccb_sample_slice(const double* matrix, int32_t m, const int32_t* input_state,
                           const double* particle_weights, int32_t n_weights, uint32_t* mt_key, int32_t* mt_pos,
                           int32_t n_samples, int32_t first, int32_t count, int32_t* samples) {
  if (!matrix || !input_state || (count > 0 && !samples) || m <= 0 || n_samples < 0 || first < 0 || count < 0 ||
      (int64_t)first + count > n_samples) {
    set_error("null pointer or bad size");
    return kErrArg;
  }
  if (m > 256) {
    set_error("the batched sampler supports at most 256 modes");
    return kErrLimit;
  }
  std::lock_guard<std::mutex> lk(g_api_mutex);
  MT19937 mt;
  int st = load_mt(mt, mt_key, mt_pos);
  if (st) return st;
  const int nw = particle_weights ? n_weights : 0;
  const char* at = getenv("BOSS_AUTOTUNE");
  if (at && at[0] == '1' && count > 0) {  // tune once per workload shape, on this call's own draws
    Context* cx = context(&st);
    if (!cx) return st;
    tune_load(cx->device);
    if (!workload_tuned(input_state, m, particle_weights, nw, mt, count)) {
      double report[8];
      if ((st = gccb_autotune_locked(cx, matrix, m, input_state, particle_weights, nw, mt, count, 3, report)))
        return st;
    }
  }
  if ((st = sample_slice_locked(matrix, m, input_state, particle_weights, nw, mt, n_samples, first, count, samples)))
    return st;
  memcpy(mt_key, mt.key, sizeof(mt.key));
  *mt_pos = mt.pos;
  return kOk;
}

int boss_gccb_autotune(const double* matrix, int32_t m, const int32_t* input_state, const double* particle_weights,
                       int32_t n_weights, const uint32_t* mt_key, const int32_t* mt_pos, int32_t n_samples,
                       int32_t reps, double* report) {
  if (!matrix || !input_state || !report || m <= 0 || n_samples <= 0 || reps <= 0) {
    set_error("null pointer or bad size");
    return kErrArg;
  }
  if (m > 256) {
    set_error("the batched sampler supports at most 256 modes");
    return kErrLimit;
  }
  std::lock_guard<std::mutex> lk(g_api_mutex);
  MT19937 mt;
  int st = load_mt(mt, mt_key, mt_pos);
  if (st) return st;
  Context* cx = context(&st);
  if (!cx) return st;
  tune_load(cx->device);
  return gccb_autotune_locked(cx, matrix, m, input_state, particle_weights, particle_weights ? n_weights : 0, mt,
                              n_samples, reps, report);
}

int boss_gccb_near_ties(int64_t* count, int32_t reset) {
  if (!count) {
    set_error("null pointer");
    return kErrArg;
  }
  std::lock_guard<std::mutex> lk(g_api_mutex);
  *count = g_gccb_near_ties;
  if (reset) g_gccb_near_ties = 0;
  return kOk;
}

int boss_perm_arithmetic(int32_t mode, int32_t* previous) {
  if (mode < -1 || mode > 1) {
    set_error("permanent arithmetic: 0 float pairs, 1 FP64, -1 query");
    return kErrArg;
  }
  std::lock_guard<std::mutex> lk(g_api_mutex);
  if (previous) *previous = g_perm_arith;
  if (mode >= 0) g_perm_arith = mode;
  return kOk;
}

int boss_minors_arithmetic(int32_t mode, int32_t* previous) {
  if (mode < -1 || mode > 1) {
    set_error("all-minors arithmetic: 0 float pairs, 1 FP64, -1 query");
    return kErrArg;
  }
  std::lock_guard<std::mutex> lk(g_api_mutex);
  if (previous) *previous = g_minors_arith;
  if (mode >= 0) g_minors_arith = mode;
  return kOk;
}

int boss_gccb_bench(const double* matrix, int32_t m, const int32_t* input_state, const double* particle_weights,
                    int32_t n_weights, uint32_t* mt_key, int32_t* mt_pos, int32_t n_samples, int32_t n_warmup,
                    int32_t n_steps, int64_t flush_bytes, double* step_ms, double* sweep_ms, double* info,
                    int32_t* samples) {
  if (!matrix || !input_state || m <= 0 || n_samples <= 0 || n_steps <= 0 || !step_ms || !sweep_ms || !info) {
    set_error("null pointer or bad size");
    return kErrArg;
  }
  if (m > 256) {
    set_error("the batched sampler supports at most 256 modes");
    return kErrLimit;
  }
  std::lock_guard<std::mutex> lk(g_api_mutex);
  MT19937 mt;
  int st = load_mt(mt, mt_key, mt_pos);
  if (st) return st;
  Draws D;
  st = predraw(input_state, m, particle_weights, particle_weights ? n_weights : 0, mt, n_samples, D);
  if (st) return st;
  const std::vector<int32_t>& L = D.L;
  const int n = D.n;
  if (n > kMaxMinorDigits || n < 1) {
    set_error("the batched sampler benchmark needs 1..32 input particles");
    return kErrLimit;
  }
  if (!std::any_of(L.begin(), L.end(), [](int32_t l) { return l > 0; })) {
    set_error("no sample keeps a particle");
    return kErrArg;
  }
  Context* cx = context(&st);
  if (!cx) return st;
  if (flush_bytes > 0 && (st = ensure(cx->misc, (size_t)flush_bytes))) return st;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaError_t e = cudaSuccess;
  // (1) the plain graph, timed per step
  GccbRun R;
  st = gccb_prepare(cx, matrix, 1, m, D, 0, R);
  for (int it = 0; !st && it < n_warmup + n_steps; ++it) {
    if (flush_bytes > 0 && (e = cudaMemsetAsync(cx->misc.ptr, it & 0xff, (size_t)flush_bytes, cx->stream)))
      break;
    cudaEventRecord(e0, cx->stream);
    if ((st = gccb_launch(cx))) break;
    cudaEventRecord(e1, cx->stream);
    if ((e = cudaEventSynchronize(e1)) != cudaSuccess) break;
    if (it >= n_warmup) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      step_ms[it - n_warmup] = ms;
    }
  }
  if (!st && e == cudaSuccess) st = gccb_collect(cx, R, samples);
  // (2) the same work with an event pair around every sweep launch: the sweep
  // kernels' share of a step (event nodes cost time, so steps are not timed here)
  GccbRun RT;
  if (!st && e == cudaSuccess) st = gccb_prepare(cx, matrix, 1, m, D, 1, RT);
  for (int it = 0; !st && e == cudaSuccess && it < n_steps; ++it) {
    if (flush_bytes > 0 && (e = cudaMemsetAsync(cx->misc.ptr, it & 0xff, (size_t)flush_bytes, cx->stream)))
      break;
    if ((st = gccb_launch(cx))) break;
    if ((e = cudaStreamSynchronize(cx->stream)) != cudaSuccess) break;
    double sw = 0.0;
    for (int k = 0; k + 1 < (int)RT.ev.size(); k += 2) {
      float x = 0.f;
      if (cudaEventElapsedTime(&x, RT.ev[k], RT.ev[k + 1]) != cudaSuccess) {
        cudaGetLastError();
        x = 0.f;
      }
      sw += x;
    }
    sweep_ms[it] = sw;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  destroy_events(RT);
  if (!st && e != cudaSuccess) st = fail_cuda(e, "bench");
  if (st) return st;
  info[0] = R.sweep_flops;
  info[6] = R.ref_flops;
  info[7] = R.ff_inst;
  info[1] = (double)R.h2d_bytes;
  info[2] = (double)R.d2h_bytes;
  info[3] = (double)R.kernels;
  info[4] = (double)R.sweeps;
  info[5] = (double)R.Lmax;
  memcpy(mt_key, mt.key, sizeof(mt.key));
  *mt_pos = mt.pos;
  return kOk;
}

// ---------------------------------------------------------------------------
// Independent instances: one (matrix, input state) per sample, pre-drawn numbers.
// ---------------------------------------------------------------------------
int boss_gccb_sample_instances(const double* matrices, int32_t n_matrices, int32_t m, const int32_t* input_states,
                               int32_t n_samples, const int32_t* randint_results, const double* uniforms,
                               int32_t stride, int32_t* samples) {
  if (!matrices || !input_states || !samples || m <= 0 || n_samples < 0 || stride < 0 ||
      (n_samples > 0 && stride > 0 && (!randint_results || !uniforms))) {
    set_error("null pointer or bad size");
    return kErrArg;
  }
  if (n_matrices != 1 && n_matrices != n_samples) {
    set_error("give one matrix, or one per sample");
    return kErrArg;
  }
  if (m > 256) {
    set_error("the batched sampler supports at most 256 modes");
    return kErrLimit;
  }
  Draws D;
  int n = 0;
  std::vector<int> ns(n_samples, 0);
  for (int s = 0; s < n_samples; ++s) {
    for (int i = 0; i < m; ++i) {
      const int v = input_states[(size_t)s * m + i];
      if (v < 0 || v > 255) {
        set_error("input occupations must be in [0, 255]");
        return kErrArg;
      }
      if (v > 1) D.binned = true;
      ns[s] += v;
    }
    n = std::max(n, ns[s]);
  }
  if (n > kMaxMinorDigits) {
    set_error("the batched sampler supports at most 32 particles per sample");
    return kErrLimit;
  }
  if (n > stride) {
    set_error("stride is below the particle count of a sample");
    return kErrArg;
  }
  D.n = n;
  const int rs = std::max(n, 1);
  D.particles.assign((size_t)n_samples * rs, 0);
  D.nparticles.assign(n_samples, 0);
  D.L.assign(n_samples, 0);
  D.idx.assign((size_t)n_samples * rs, 0);
  D.u.assign((size_t)n_samples * rs, 0.0);
  for (int s = 0; s < n_samples; ++s) {
    int p = 0;
    for (int i = 0; i < m; ++i)
      for (int c = 0; c < input_states[(size_t)s * m + i]; ++c) D.particles[(size_t)s * rs + p++] = (uint8_t)i;
    D.nparticles[s] = (uint8_t)ns[s];
    D.L[s] = ns[s];
    for (int k = 0; k < ns[s]; ++k) {
      const int r = randint_results[(size_t)s * stride + k];
      if (r < 0 || r >= ns[s] - k) {
        set_error("a randint result is outside [0, particles left)");
        return kErrArg;
      }
      D.idx[(size_t)s * rs + k] = (uint8_t)r;
      D.u[(size_t)s * rs + k] = uniforms[(size_t)s * stride + k];
    }
  }
  D.n = rs;
  memset(samples, 0, sizeof(int32_t) * (size_t)n_samples * m);
  if (n == 0) return kOk;
  std::lock_guard<std::mutex> lk(g_api_mutex);
  int st;
  Context* cx = context(&st);
  if (!cx) return st;
  return run_gccb(cx, matrices, n_matrices, m, D, samples);
}

// numpy legacy choice(range(len(p)), p=p): cdf = cumsum(p) / its last entry, one
// random_sample, searchsorted(..., 'right').
static std::vector<double> choice_cdf(const double* p, int n) {
  std::vector<double> cdf(n);
  double acc = 0.0;
  for (int i = 0; i < n; ++i) cdf[i] = acc = acc + p[i];
  const double last = cdf[n - 1];
  for (int i = 0; i < n; ++i) cdf[i] /= last;
  return cdf;
}
static int choice_draw(MT19937& mt, const std::vector<double>& cdf) {
  const double u = mt.next_double();
  return (int)(std::upper_bound(cdf.begin(), cdf.end(), u) - cdf.begin());
}
// The C&C-B steps of one lossless sample: per particle randint(0, left), then
// numpy.random.choice's random_sample (generalized_cliffords_b_simulation_strategy.py:97-110).
static void gccb_draws(MT19937& mt, int particles, int32_t* ri, double* uu) {
  for (int k = 0; k < particles; ++k) {
    const uint32_t left = (uint32_t)(particles - k);
    ri[k] = (int32_t)mt.bounded(left, mask_for(left));
    uu[k] = mt.next_double();
  }
}

int boss_bobs_uniform_predraw(uint32_t* mt_key, int32_t* mt_pos, int32_t n_samples, int32_t m, int32_t k,
                              const int32_t* exact_parts, const double* exact_weights, int32_t n_exact,
                              const int32_t* approx_parts, const double* approx_weights, int32_t n_approx,
                              int32_t stride, int32_t* input_states, double* phase_uniforms, int32_t* permutations,
                              int32_t* randint_results, double* uniforms) {
  if (!mt_key || !mt_pos || n_samples < 0 || m <= 0 || k < 0 || k > m || n_exact <= 0 || n_approx <= 0 ||
      !exact_weights || !approx_weights || !input_states || !permutations || stride < 0) {
    set_error("null pointer or bad size");
    return kErrArg;
  }
  MT19937 mt;
  int st = load_mt(mt, mt_key, mt_pos);
  if (st) return st;
  const int ma = m - k;  // approximated modes
  const std::vector<double> cdf_a = choice_cdf(approx_weights, n_approx), cdf_e = choice_cdf(exact_weights, n_exact);
  for (int s = 0; s < n_samples; ++s) {
    // lossy_state_approximated_simulation_strategy.py:312-332: approximated part first
    const int ia = choice_draw(mt, cdf_a);
    const int ie = choice_draw(mt, cdf_e);
    int32_t* in = input_states + (size_t)s * m;
    int particles = 0;
    for (int i = 0; i < k; ++i) particles += (in[i] = exact_parts[(size_t)ie * k + i]);
    for (int i = 0; i < ma; ++i) particles += (in[k + i] = approx_parts[(size_t)ia * ma + i]);
    if (particles > stride) {
      set_error("stride is below the particle count of a sample");
      return kErrArg;
    }
    // :348-362: the random phases are drawn before the column permutation
    for (int i = 0; i < ma; ++i) phase_uniforms[(size_t)s * ma + i] = mt.next_double();
    int32_t* perm = permutations + (size_t)s * m;
    for (int i = 0; i < m; ++i) perm[i] = i;
    for (int i = m - 1; i >= 1; --i) {  // numpy's legacy shuffle
      const uint32_t j = mt.bounded((uint32_t)i + 1u, mask_for((uint32_t)i + 1u));
      std::swap(perm[i], perm[j]);
    }
    gccb_draws(mt, particles, randint_results + (size_t)s * stride, uniforms + (size_t)s * stride);
  }
  memcpy(mt_key, mt.key, sizeof(mt.key));
  *mt_pos = mt.pos;
  return kOk;
}

int boss_bobs_nonuniform_predraw(uint32_t* mt_key, int32_t* mt_pos, int32_t n_samples, int32_t m,
                                 const int32_t* base_state, int32_t approximated_modes, int32_t approximated_particles,
                                 const double* loss_weights, int32_t max_occupation, int32_t lossy, int32_t stride,
                                 int32_t* input_states, double* phase_uniforms, int32_t* randint_results,
                                 double* uniforms) {
  if (!mt_key || !mt_pos || n_samples < 0 || m <= 0 || !base_state || approximated_modes < 0 ||
      approximated_modes > m || max_occupation < 0 || !input_states || stride < 0 || (lossy && !loss_weights)) {
    set_error("null pointer or bad size");
    return kErrArg;
  }
  MT19937 mt;
  int st = load_mt(mt, mt_key, mt_pos);
  if (st) return st;
  const int ka = approximated_modes;
  const int W = max_occupation + 1;  // loss_weights: row o = binomial weights of o particles
  std::vector<int32_t> state(m);
  for (int s = 0; s < n_samples; ++s) {
    // nonuniform_losses_approximation_strategy.py:280-294
    for (int i = 0; i < m; ++i) state[i] = base_state[i];
    if (ka > 0) state[mt.bounded((uint32_t)ka, mask_for((uint32_t)ka))] = approximated_particles;
    int32_t* in = input_states + (size_t)s * m;
    int particles = 0;
    for (int i = 0; i < m; ++i) {  // :298-329, the module's own choice()
      const int occ = state[i];
      int v = occ;
      if (lossy && occ > 0) {
        if (occ > max_occupation) {
          set_error("an occupation exceeds the loss-weight table");
          return kErrArg;
        }
        const double r = mt.next_double();
        double acc = 0.0;
        v = -1;
        for (int q = 0; q <= occ; ++q) {
          acc += loss_weights[(size_t)occ * W + q];
          if (acc > r) {
            v = q;
            break;
          }
        }
        if (v < 0) {
          set_error("loss weights sum below the random number");
          return kErrArg;
        }
      }
      particles += (in[i] = v);
    }
    if (particles > stride) {
      set_error("stride is below the particle count of a sample");
      return kErrArg;
    }
    for (int i = 0; i < ka; ++i) phase_uniforms[(size_t)s * ka + i] = mt.next_double();
    gccb_draws(mt, particles, randint_results + (size_t)s * stride, uniforms + (size_t)s * stride);
  }
  memcpy(mt_key, mt.key, sizeof(mt.key));
  *mt_pos = mt.pos;
  return kOk;
}

}  // extern "C"
