// engine.cu -- GB300 (sm_103a) CT-HYB pair-move engine.
//
// One warp advances one Markov chain through the proposal loop of the
// w2dynamics Fortran module (CTQMC.F90 ctqmc_warmup / ctqmc_measure ->
// StepAdd / StepRem), so that a launch of N warps advances N independent
// chains; a batch of one chain is the plain drop-in form.
//
// Per chain, in HBM:
//   * a Mersenne-twister state that reproduces, draw for draw, the
//     reference's std::mt19937 + uniform_real_distribution<double> +
//     uniform_int_distribution<int> stream (src/mtrng/random.cc:35-78), so a
//     chain seeded with s makes exactly the proposals of the reference run
//     seeded with s;
//   * the time-ordered operator array and, per flavour, the sorted creator
//     and annihilator times (ranks = the FPos of Trace.F90:4275-4500);
//   * per flavour the inverse hybridisation matrix M in "slot" order: rows
//     and columns stay where they were appended, so the Sherman-Morrison
//     grow/shrink of MatrixUpdate.F90:392-482 needs no row/column shifting;
//   * a binary tree over 2^L equal time bins of [0, beta): each node holds,
//     for every superstate, the superstate it is mapped to across the node's
//     time span, and (density-density models) for every eigenstate the
//     target state, log-weight and sign of the time-ordered product of
//     propagators and c/c+ operators inside the span.  A pair move rebuilds
//     at most two leaves and their ancestors (O(L) nodes) in the inactive
//     half of a double buffer; acceptance flips the active bits.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/cthyb_gpu.h"
#include "engine.cuh"
#include "model.h"

namespace cthyb {

// Code size of the proposal path decides performance: with ~30 warps per SM
// at different points of a fully inlined path the instruction cache
// thrashes, so the larger building blocks exist once.
#ifdef CTHYB_INLINE_ALL
#define NOINL __forceinline__
#else
#define NOINL __noinline__
#endif

#ifdef CTHYB_PROFILE
#define PROF_START() long long prof_t0_ = clock64()
#define PROF_MARK(i)                                      \
  do {                                                    \
    long long t_ = clock64();                             \
    if (c.lane == 0) c.h->prof[i] += t_ - prof_t0_;       \
    prof_t0_ = t_;                                        \
  } while (0)
#else
#define PROF_START() \
  do {               \
  } while (0)
#define PROF_MARK(i) \
  do {               \
  } while (0)
#endif

// ---------------------------------------------------------------------------
// Chain context (all lanes hold the same values).
struct Ctx {
  const DModel* m;
  const DGroup* g;
  Hdr* h;
  uint32_t* mt;
  double* optau;
  int* opcode;
  double* srt_tau;
  short* srt_slot;
  double* slot_tau;
  double* M;
  char* tree;
  unsigned char* act;
  int* bstart;  // [2^L + 1] index of the first operator of each time bin
  double* scr;
  double* btau[2];
  double* bdt[2];  // time steps before each gathered operator and to the bin end
  int* bcode[2];
  double* gtau;
  double* histo;
  double* dm;
  double* dense;
  cthyb_record* log;
  cthyb_record* rec;  // per-warp record under construction (shared memory)
  int lane, mono, kcap, chain;
  // next tempered generator outputs: lane i holds output mtbase + i;
  // mtpos is the next unread position, mtcnt the valid count
  uint32_t mtbuf;
  int mtbase, mtpos, mtcnt;
};

__device__ __forceinline__ double* srt_ptr(const Ctx& c, int f, int ca) {
  return c.srt_tau + (size_t)(f * 2 + ca) * c.kcap;
}
__device__ __forceinline__ short* sslot_ptr(const Ctx& c, int f, int ca) {
  return c.srt_slot + (size_t)(f * 2 + ca) * c.kcap;
}
__device__ __forceinline__ double* stau_ptr(const Ctx& c, int f, int ca) {
  return c.slot_tau + (size_t)(f * 2 + ca) * c.kcap;
}
__device__ __forceinline__ double* M_ptr(const Ctx& c, int f) {
  return c.M + (size_t)f * c.kcap * c.kcap;
}

__device__ __forceinline__ void set_status(Ctx& c, int st) {
  if (c.lane == 0 && c.h->status == ST_OK) c.h->status = st;
  __syncwarp();
}

// ---------------------------------------------------------------------------
// Warp reductions
__device__ __forceinline__ double wsum(double x) {
#pragma unroll
  for (int o = 16; o; o >>= 1) x += __shfl_xor_sync(FULL, x, o);
  return x;
}
__device__ __forceinline__ double wmax(double x) {
#pragma unroll
  for (int o = 16; o; o >>= 1) x = fmax(x, __shfl_xor_sync(FULL, x, o));
  return x;
}
__device__ __forceinline__ int wsumi(int x) {
#pragma unroll
  for (int o = 16; o; o >>= 1) x += __shfl_xor_sync(FULL, x, o);
  return x;
}

// ---------------------------------------------------------------------------
// Mersenne twister MT19937 (Matsumoto & Nishimura 1998), warp-cooperative
// state regeneration; the uniform double follows the C++ standard's
// generate_canonical with two 32-bit draws, the bounded integer Lemire's
// nearly-divisionless method (ACM TOMACS 29(1), 2019) -- the algorithms of
// the standard library used by src/mtrng/random.cc.
__device__ NOINL void mt_twist(uint32_t* mt, int lane) {
  for (int base = 0; base < 624; base += 32) {
    int i = base + lane;
    bool on = i < 624;
    uint32_t a = 0, b = 0, cc = 0;
    if (on) {
      a = mt[i];
      b = mt[i + 1 < 624 ? i + 1 : 0];
      cc = mt[i + 397 < 624 ? i + 397 : i + 397 - 624];
    }
    __syncwarp();
    if (on) {
      uint32_t y = (a & 0x80000000u) | (b & 0x7fffffffu);
      mt[i] = cc ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
    }
    __syncwarp();
  }
}
__device__ __forceinline__ uint32_t mt_temper(uint32_t y) {
  y ^= y >> 11;
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  y ^= y >> 18;
  return y;
}
// Load the 32 outputs starting at state index `from` (twisting first when
// the state is exhausted) into the lanes' buffer.
__device__ NOINL void mt_refill(Ctx& c, int from) {
  if (from >= 624) {
    mt_twist(c.mt, c.lane);
    from = 0;
  }
  c.mtbase = from;
  c.mtcnt = min(32, 624 - from);
  c.mtpos = 0;
  int i = from + c.lane;
  c.mtbuf = i < 624 ? mt_temper(c.mt[i]) : 0u;
}
__device__ __forceinline__ uint32_t mt_next(Ctx& c) {
  if (c.mtpos >= c.mtcnt) mt_refill(c, c.mtbase + c.mtcnt);
  uint32_t y = __shfl_sync(FULL, c.mtbuf, c.mtpos);
  c.mtpos++;
  return y;
}
// generator position (index of the next output) for the chain header
__device__ __forceinline__ int mt_index(const Ctx& c) { return c.mtbase + c.mtpos; }
__device__ __forceinline__ double grnd(Ctx& c) {
  uint32_t a = mt_next(c);
  uint32_t b = mt_next(c);
  // generate_canonical: RN(a + b 2^32) / 2^64.  a + b 2^32 is the 64-bit
  // integer v, so one correctly rounded u64->f64 conversion gives the sum,
  // and the scaling by 2^-64 is an exponent shift (exact, v >= 1).
  unsigned long long v = ((unsigned long long)b << 32) | a;
  if (v == 0ull) return 0.0;
  // round v to 53 bits (to nearest, ties to even) with integer operations
  // and build the double v * 2^-64 directly: exponent -1 - lz, carry of the
  // rounding into the exponent field included (keeps the FP64 pipe free)
  const int lz = __clzll(v);
  const unsigned long long m = v << lz;  // leading one at bit 63
  unsigned long long mant = m >> 11;     // 53 bits with the hidden one
  const unsigned long long rest = m & 0x7FFull;
  if (rest > 0x400ull || (rest == 0x400ull && (mant & 1ull))) ++mant;
  long long bits = (long long)(((unsigned long long)(1022 - lz) << 52) + (mant - (1ull << 52)));
  if (bits >= 0x3FF0000000000000ll) bits = 0x3FEFFFFFFFFFFFFFll;  // 1.0 -> nextafter(1, 0)
  return __longlong_as_double(bits);
}
__device__ __forceinline__ int randint(Ctx& c, int lo, int hi) {
  uint32_t range = (uint32_t)(hi - lo) + 1u;
  uint64_t prod = (uint64_t)mt_next(c) * range;
  uint32_t low = (uint32_t)prod;
  if (low < range) {
    uint32_t thr = (0u - range) % range;
    int guard = 0;
    while (low < thr) {
      prod = (uint64_t)mt_next(c) * range;
      low = (uint32_t)prod;
      if (++guard > 256) {
        set_status(c, ST_INTERNAL);
        break;
      }
    }
  }
  return lo + (int)(prod >> 32);
}
__device__ void mt_seed(uint32_t* mt, uint32_t seed, int lane) {
  if (lane == 0) {
    mt[0] = seed;
    for (int i = 1; i < 624; ++i) mt[i] = 1812433253u * (mt[i - 1] ^ (mt[i - 1] >> 30)) + (uint32_t)i;
  }
  __syncwarp();
}

// ---------------------------------------------------------------------------
// Warp 32-ary searches on sorted arrays of non-negative doubles.  For
// x >= 0 the IEEE-754 order equals the order of the bit patterns read as
// signed 64-bit integers, so the comparisons run on the integer pipes
// (exact, and FP64 throughput on GB300 is scarce).
__device__ __forceinline__ long long tkey(double x) {
  long long b = __double_as_longlong(x);
  return b == (long long)0x8000000000000000ll ? 0ll : b;  // -0.0 -> +0.0
}
// first index i in [0,n) with !(a[i] < x)   (lower bound)
__device__ NOINL int wlb(const double* ad, int n, double x, int lane) {
  const long long* a = (const long long*)ad;
  const long long xb = tkey(x);
  int lo = 0, hi = n;
  while (hi - lo > 32) {
    int step = (hi - lo + 31) >> 5;
    int p = lo + lane * step;
    bool pr = (p < hi) && (a[p] < xb);
    int cnt = __popc(__ballot_sync(FULL, pr));
    if (cnt == 0) {
      hi = lo;
      break;
    }
    int pl = lo + (cnt - 1) * step, pn = lo + cnt * step;
    lo = pl + 1;
    hi = min(pn, hi);
  }
  if (hi > lo) {
    int p = lo + lane;
    bool pr = (p < hi) && (a[p] < xb);
    lo += __popc(__ballot_sync(FULL, pr));
  }
  return lo;
}
// first index i with a[i] > x   (upper bound)
__device__ NOINL int wub(const double* ad, int n, double x, int lane) {
  const long long* a = (const long long*)ad;
  const long long xb = tkey(x);
  int lo = 0, hi = n;
  while (hi - lo > 32) {
    int step = (hi - lo + 31) >> 5;
    int p = lo + lane * step;
    bool pr = (p < hi) && (a[p] <= xb);
    int cnt = __popc(__ballot_sync(FULL, pr));
    if (cnt == 0) {
      hi = lo;
      break;
    }
    int pl = lo + (cnt - 1) * step, pn = lo + cnt * step;
    lo = pl + 1;
    hi = min(pn, hi);
  }
  if (hi > lo) {
    int p = lo + lane;
    bool pr = (p < hi) && (a[p] <= xb);
    lo += __popc(__ballot_sync(FULL, pr));
  }
  return lo;
}
// sequential (single-thread) versions for per-lane use
__device__ __forceinline__ int slb(const double* ad, int n, double x) {
  const long long* a = (const long long*)ad;
  const long long xb = tkey(x);
  int lo = 0, hi = n;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (a[mid] < xb) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}
__device__ __forceinline__ int sub(const double* ad, int n, double x) {
  const long long* a = (const long long*)ad;
  const long long xb = tkey(x);
  int lo = 0, hi = n;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (a[mid] <= xb) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}
__device__ __forceinline__ bool teq(double a, double b) { return tkey(a) == tkey(b); }

// ---------------------------------------------------------------------------
// Hybridisation function: the linear interpolation of get_HybrF,
// Trace.F90:1014-1033.  The grid coordinate is tau * ((Nftau - 1) / beta)
// (the reference divides first: tau / beta * (Nftau - 1)) and the
// interpolation is one fused multiply-add, so the value agrees with the
// reference's to within a few units in the last place -- far inside the
// 1e-10 tolerance of the ratios -- at one FP64 multiply instead of a
// division per call.
__device__ __forceinline__ double hybrf(const Ctx& c, double tau, int f) {
  const DGroup& g = *c.g;
  // tau is a difference of distinct times, never -0.0, so the sign bit
  // decides the antiperiodic branch
  const long long neg = __double_as_longlong(tau) & (long long)0x8000000000000000ll;
  if (neg) tau = tau + g.beta;
  double n = tau * g.hscale;  // hscale = (Nftau - 1) / beta
  int in = (int)n;
  double fr = n - (double)in;
  int i = min(max(in, 0), g.nftau - 2);
  const double* F = g.hybr + (size_t)f * g.nftau;
  double f0 = __ldg(F + i), f1 = __ldg(F + i + 1);
  double v = fma(fr, f1 - f0, f0);
  return __longlong_as_double(__double_as_longlong(v) ^ neg);
}

// ---------------------------------------------------------------------------
// Window (Trace.F90:1608-1754)
__device__ NOINL void set_window_bounds(Ctx& c) {
  Hdr& h = *c.h;
  if (c.lane == 0 && h.num_windows > 1) {
    h.tauwin_min = __dmul_rn(__ddiv_rn((double)h.window_position, (double)(h.num_windows + 1)), c.g->beta);
    h.tauwin_max = __dmul_rn(__ddiv_rn((double)(h.window_position + 2), (double)(h.num_windows + 1)), c.g->beta);
  }
  __syncwarp();
}
__device__ NOINL void init_window(Ctx& c, double tdm) {
  Hdr& h = *c.h;
  if (c.lane == 0) {
    h.window_position = 0;
    if (tdm > 0.0) {
      h.taudiff_max = tdm;
      int nw = (int)floor(c.g->beta / tdm) - 1;
      h.num_windows = nw > 1 ? nw : 1;
      h.tauwin_min = __dmul_rn(__ddiv_rn(0.0, (double)(h.num_windows + 1)), c.g->beta);
      h.tauwin_max = __dmul_rn(__ddiv_rn(2.0, (double)(h.num_windows + 1)), c.g->beta);
    } else {
      h.taudiff_max = c.g->beta;
      h.num_windows = 1;
      h.tauwin_min = 0.0;
      h.tauwin_max = c.g->beta;
    }
    h.npairs = -1;
  }
  __syncwarp();
}
__device__ NOINL void shift_window(Ctx& c) {
  Hdr& h = *c.h;
  if (h.num_windows > 1) {
    if (c.lane == 0) {
      h.window_position += 1;
      if (h.window_position == h.num_windows) h.window_position = 0;
      h.npairs = -1;
    }
    __syncwarp();
    set_window_bounds(c);
  } else {
    if (c.lane == 0) h.window_position = 0;
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------
// Pair counting (ensure_valid_NPairs_diag / update_NPairs_diag,
// Trace.F90:1756-1922) on the sorted per-flavour arrays.
// Later partners of an operator at t: opposite-CA times u with
// t < u <= min(win_max, t + tdm).
__device__ __forceinline__ int cnt_later(const double* opp, int n, double t, double wmax, double tdm) {
  double hi = fmin(wmax, __dadd_rn(t, tdm));
  int a = sub(opp, n, t), b = sub(opp, n, hi);
  return b > a ? b - a : 0;
}
// Earlier partners: max(win_min, t - tdm) <= u < t.
__device__ __forceinline__ int cnt_earlier(const double* opp, int n, double t, double wmin, double tdm) {
  double lo = fmax(wmin, __dsub_rn(t, tdm));
  int a = slb(opp, n, lo), b = slb(opp, n, t);
  return b > a ? b - a : 0;
}
// Partners of two operators (times t1, t2) among the opposite-CA lists
// opp1, opp2 (n1, n2 entries): cnt_later + cnt_earlier of each, the eight
// binary searches run by lanes 0..7 at once instead of one after the
// other.  Warp-uniform result.
__device__ __forceinline__ int partner_counts(const Ctx& c, const double* opp1, int n1, double t1,
                                              const double* opp2, int n2, double t2, double wmin, double wmax,
                                              double tdm) {
  const int l = c.lane;
  int r = 0;
  if (l < 8) {
    const bool second = l >= 4;
    const double* opp = second ? opp2 : opp1;
    const int n = second ? n2 : n1;
    const double t = second ? t2 : t1;
    const int q = l & 3;
    if (q == 0) r = sub(opp, n, t);                               // later: lower end
    else if (q == 1) r = sub(opp, n, fmin(wmax, __dadd_rn(t, tdm)));  // later: upper end
    else if (q == 2) r = slb(opp, n, fmax(wmin, __dsub_rn(t, tdm)));  // earlier: lower end
    else r = slb(opp, n, t);                                      // earlier: upper end
  }
  const int up = __shfl_down_sync(FULL, r, 1);
  int d = (l < 8 && (l & 1) == 0 && up > r) ? up - r : 0;
  d += __shfl_down_sync(FULL, d, 2);
  d += __shfl_down_sync(FULL, d, 4);
  return __shfl_sync(FULL, d, 0);
}
__device__ NOINL int count_npairs(Ctx& c) {
  Hdr& h = *c.h;
  int K = h.K;
  int start = wlb(c.optau, K, h.tauwin_min, c.lane);
  int tot = 0;
  for (int i = start + c.lane; i < K; i += 32) {
    double t = c.optau[i];
    if (t > h.tauwin_max) continue;
    int code = c.opcode[i], f = code >> 1, ca = code & 1;
    tot += cnt_later(srt_ptr(c, f, 1 - ca), h.k[f], t, h.tauwin_max, h.taudiff_max);
  }
  return wsumi(tot);
}

// ---------------------------------------------------------------------------
// Configuration sign (get_Sign with get_BlockSign and get_permaltca,
// Trace.F90:3479-3621).  BlockSign counts, for each operator, the
// operators after it whose flavour index 2b+s is smaller; permaltca counts
// for each creator the operators of its flavour after it, plus one if the
// number of pairs is odd.
__device__ NOINL double config_sign(Ctx& c) {
  Hdr& h = *c.h;
  const int K = h.K, nf = c.m->nf;
  const unsigned lt = (1u << c.lane) - 1u;
  int run[NFMAX];
#pragma unroll
  for (int g = 0; g < NFMAX; ++g) run[g] = 0;
  int inv = 0, alt = 0;
  for (int base = 0; base < K; base += 32) {
    int i = base + c.lane;
    int code = i < K ? c.opcode[i] : -2;
    int f = code >> 1;
    bool cre = i < K && (code & 1) == 0;
#pragma unroll
    for (int g = 0; g < NFMAX; ++g) {
      if (g >= nf) break;
      unsigned msk = __ballot_sync(FULL, f == g);
      int before = run[g] + __popc(msk & lt);  // operators of flavour g before i
      if (i < K) {
        if (g > f) inv += before;
        if (g == f && cre) alt += 2 * h.k[g] - before - 1;  // of flavour g after i
      }
      run[g] += __popc(msk);
    }
  }
  inv = wsumi(inv & 1) & 1;
  alt = wsumi(alt & 1) & 1;
  if ((K / 2) % 2 == 1) alt ^= 1;
  double bs = inv ? -1.0 : 1.0, pa = alt ? -1.0 : 1.0;
  return h.trace_sign * h.det_sign * bs * pa;
}

// ---------------------------------------------------------------------------
// Time-bin tree
struct Mod {
  int type;         // 0 none, 1 insert, 2 remove
  double t1, t2;    // inserted times (t1 < t2)
  int c1, c2;       // inserted codes
  int ix, iy;       // removed indices (ix < iy)
  int b1, b2;       // affected leaves
  int n1, n2;       // gathered operator counts of leaves b1, b2 (buffers 0, 1)
  int p1, p2;       // insertion: lower bounds of t1, t2 in the operator array
};

// Bin edges beta * j / 2^L (tabulated per group) and the bin of a time by
// an integer search over their order keys (no FP64 work).
__device__ __forceinline__ double bin_edge(const Ctx& c, int j) { return c.g->edges[j]; }
__device__ __forceinline__ int bin_of(const Ctx& c, double t) {
  const long long tb = tkey(t);
  const long long* ek = c.g->ekeys;
  int lo = 0, hi = 1 << c.g->L;  // the bin is the last j in [lo, hi) with ek[j] <= tb
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (ek[mid] <= tb) lo = mid;
    else hi = mid;
  }
  return lo;
}
__device__ __forceinline__ char* node_base(const Ctx& c, int n, int slot) {
  return c.tree + ((size_t)n * 2 + slot) * c.g->node_bytes;
}
__device__ __forceinline__ double* node_lw(const Ctx& c, int n, int slot) {
  return (double*)node_base(c, n, slot);
}
__device__ __forceinline__ uint16_t* node_tg(const Ctx& c, int n, int slot) {
  return (uint16_t*)(node_base(c, n, slot) + (size_t)c.m->ns * 8);
}
__device__ __forceinline__ int16_t* node_ss(const Ctx& c, int n, int slot) {
  return (int16_t*)(node_base(c, n, slot) + (c.mono ? (size_t)c.m->ns * 10 : 0));
}
__device__ __forceinline__ bool node_mod(const Ctx& c, const Mod& md, int n) {
  if (md.type == 0) return false;
  int L = c.g->L;
  int d = 31 - __clz(n);
  int n1 = ((1 << L) + md.b1) >> (L - d), n2 = ((1 << L) + md.b2) >> (L - d);
  return n == n1 || n == n2;
}
// slot holding the proposed content of node n
__device__ __forceinline__ int node_slot(const Ctx& c, const Mod& md, int n) {
  int a = c.act[n];
  return node_mod(c, md, n) ? 1 - a : a;
}

// Gather the operators of bin b of the proposed configuration into
// btau/bcode; returns their number.
__device__ NOINL int gather_bin(Ctx& c, const Mod& md, int b, int buf) {
  double* btau = c.btau[buf];
  int* bcode = c.bcode[buf];
  const int nb = 1 << c.g->L;
  double e0 = bin_edge(c, b), e1 = b + 1 < nb ? bin_edge(c, b + 1) : 0.0;
  const int lo = c.bstart[b], hi = c.bstart[b + 1];
  bool in1 = false, in2 = false;
  if (md.type == 1) {
    in1 = bin_of(c, md.t1) == b;
    in2 = bin_of(c, md.t2) == b;
  }
  int nrem = 0;
  if (md.type == 2) nrem = (md.ix >= lo && md.ix < hi) + (md.iy >= lo && md.iy < hi);
  for (int j = lo + c.lane; j < hi; j += 32) {
    double t = c.optau[j];
    int code = c.opcode[j];
    int r = j - lo;
    if (md.type == 1) {
      r += (in1 && md.t1 < t) + (in2 && md.t2 < t);
    } else if (md.type == 2) {
      if (j == md.ix || j == md.iy) continue;
      r -= (md.ix >= lo && md.ix < j) + (md.iy >= lo && md.iy < j);
    }
    btau[r] = t;
    bcode[r] = code;
  }
  int n = hi - lo - nrem;
  if (md.type == 1) {
    // positions of the inserted operators
    int p1 = 0, p2 = 0;
    if (in1) p1 = wlb(c.optau + lo, hi - lo, md.t1, c.lane);
    if (in2) p2 = wlb(c.optau + lo, hi - lo, md.t2, c.lane) + (in1 ? 1 : 0);
    if (c.lane == 0) {
      if (in1) {
        btau[p1] = md.t1;
        bcode[p1] = md.c1;
      }
      if (in2) {
        btau[p2] = md.t2;
        bcode[p2] = md.c2;
      }
    }
    n += in1 + in2;
  }
  __syncwarp();
  // time steps: before operator j from the previous one (bin start for j=0),
  // and from the last operator to the bin end (index n)
  double* bdt = c.bdt[buf];
  double t1 = b + 1 < nb ? e1 : c.g->beta;
  for (int j = c.lane; j <= n; j += 32) {
    double prev = j > 0 ? btau[j - 1] : e0;
    double cur = j < n ? btau[j] : t1;
    bdt[j] = cur - prev;
  }
  __syncwarp();
  return n;
}

// The operators of the proposal's one or two leaves (bins md.b1, md.b2) of
// the proposed configuration gathered together into buffers 0 and 1, with
// their time steps: the same buffers as gather_bin for each bin, with one
// pass over both bins instead of one after the other.  Leaf 0 holds t1 (and
// t2 when both are in one bin), leaf 1 holds t2; the inserted operators go
// to their lower bounds md.p1, md.p2 in the operator array.
__device__ NOINL void gather_leaves(Ctx& c, Mod& md, int nleaf) {
  const int nb = 1 << c.g->L;
  const int lo0 = c.bstart[md.b1], hi0 = c.bstart[md.b1 + 1];
  const int lo1 = c.bstart[md.b2], hi1 = c.bstart[md.b2 + 1];
  const int len0 = hi0 - lo0, len1 = nleaf > 1 ? hi1 - lo1 : 0;
  const bool ins = md.type == 1, rem = md.type == 2;
  for (int t = c.lane; t < len0 + len1; t += 32) {
    const int q = t >= len0 ? 1 : 0;
    const int lo = q ? lo1 : lo0;
    const int j = lo + t - q * len0;
    const double tau = c.optau[j];
    const int code = c.opcode[j];
    int r = j - lo;
    if (ins) {
      r += (q == 0 && md.t1 < tau) + ((q == 1 || nleaf == 1) && md.t2 < tau);
    } else if (rem) {
      if (j == md.ix || j == md.iy) continue;
      r -= (md.ix >= lo && md.ix < j) + (md.iy >= lo && md.iy < j);
    }
    c.btau[q][r] = tau;
    c.bcode[q][r] = code;
  }
  int n0 = len0, n1 = len1;
  if (rem) {
    n0 -= (md.ix >= lo0 && md.ix < hi0) + (md.iy >= lo0 && md.iy < hi0);
    if (nleaf > 1) n1 -= (md.ix >= lo1 && md.ix < hi1) + (md.iy >= lo1 && md.iy < hi1);
  }
  if (ins) {
    if (c.lane == 0) {
      c.btau[0][md.p1 - lo0] = md.t1;
      c.bcode[0][md.p1 - lo0] = md.c1;
      const int q2 = nleaf > 1 ? 1 : 0;
      const int p2 = md.p2 - (q2 ? lo1 : lo0) + (q2 ? 0 : 1);
      c.btau[q2][p2] = md.t2;
      c.bcode[q2][p2] = md.c2;
    }
    if (nleaf > 1) {
      n0 += 1;
      n1 += 1;
    } else {
      n0 += 2;
    }
  }
  md.n1 = n0;
  md.n2 = nleaf > 1 ? n1 : n0;
  __syncwarp();
  // time steps: before operator j from the previous one (bin start for
  // j = 0), and from the last operator to the bin end (index n)
  const int m0 = n0 + 1, tot = m0 + (nleaf > 1 ? n1 + 1 : 0);
  for (int t = c.lane; t < tot; t += 32) {
    const int q = t >= m0 ? 1 : 0, j = t - q * m0, n = q ? n1 : n0, b = q ? md.b2 : md.b1;
    const double* bt = c.btau[q];
    const double prev = j > 0 ? bt[j - 1] : bin_edge(c, b);
    const double cur = j < n ? bt[j] : (b + 1 < nb ? bin_edge(c, b + 1) : c.g->beta);
    c.bdt[q][j] = cur - prev;
  }
  __syncwarp();
}

// Leaf of bin b from the gathered operators (n of them), written to `slot`:
// superstate map (do_ss) and/or state map (do_states).
__device__ __forceinline__ void leaf_body(Ctx& c, int b, int n, int slot, bool do_ss, bool do_states, int buf) {
  const DModel& m = *c.m;
  const int* bcode = c.bcode[buf];
  const int L = c.g->L, nb = 1 << L, node = nb + b;
  int16_t* ss = node_ss(c, node, slot);
  for (int s = c.lane; do_ss && s < m.nss; s += 32) {
    int cur = s;
    for (int j = 0; j < n && cur >= 0; ++j) {
      int code = bcode[j];
      cur = m.connect[((size_t)cur * m.nf + (code >> 1)) * 2 + (code & 1)];
    }
    ss[s] = (int16_t)cur;
  }
  if (do_states && c.mono) {
    const double* bdt = c.bdt[buf];
    double* lw = node_lw(c, node, slot);
    uint16_t* tg = node_tg(c, node, slot);
    if (m.ns <= 16 * c.kcap) {
      // Integer walk first (target state and sign of every start state),
      // then the log weights of the surviving start states only, one per
      // lane: the FP64 work scales with the survivors, not with the states.
      int16_t* surv = (int16_t*)c.scr;  // the determinant scratch is idle here
      int nsurv = 0;
      for (int s0 = 0; s0 < m.ns; s0 += 32) {
        const int s = s0 + c.lane;
        int cur = s < m.ns ? s : -1, neg = 0;
        for (int j = 0; j < n && cur >= 0; ++j) {
          const size_t idx = (size_t)bcode[j] * m.ns + cur;
          neg ^= m.mono_neg[idx];
          cur = m.mono_tgt[idx];
        }
        if (s < m.ns) {
          tg[s] = cur >= 0 ? (uint16_t)(cur | (neg << 15)) : (uint16_t)0x7fff;
          if (cur < 0) lw[s] = -DHUGE;
        }
        const unsigned bal = __ballot_sync(FULL, cur >= 0);
        if (cur >= 0) surv[nsurv + __popc(bal & ((1u << c.lane) - 1u))] = (int16_t)s;
        nsurv += __popc(bal);
      }
      __syncwarp();
      for (int q = c.lane; q < nsurv; q += 32) {
        const int s = surv[q];
        int cur = s;
        double l = 0.0;
        for (int j = 0; j < n; ++j) {
          l = fma(-m.evs[cur], bdt[j], l);
          const size_t idx = (size_t)bcode[j] * m.ns + cur;
          if (!m.mono_lv0) l += m.mono_lv[idx];
          cur = m.mono_tgt[idx];
        }
        lw[s] = fma(-m.evs[cur], bdt[n], l);
      }
    } else {
      for (int s = c.lane; s < m.ns; s += 32) {
        int cur = s;
        double l = 0.0;
        int neg = 0;
        for (int j = 0; j < n; ++j) {
          l = fma(-m.evs[cur], bdt[j], l);
          size_t idx = (size_t)bcode[j] * m.ns + cur;
          int nx = m.mono_tgt[idx];
          if (nx < 0) {
            cur = -1;
            break;
          }
          l += m.mono_lv[idx];
          neg ^= m.mono_neg[idx];
          cur = nx;
        }
        if (cur >= 0) {
          l = fma(-m.evs[cur], bdt[n], l);
          tg[s] = (uint16_t)(cur | (neg << 15));
          lw[s] = l;
        } else {
          tg[s] = 0x7fff;
          lw[s] = -DHUGE;
        }
      }
    }
  }
  __syncwarp();
}

// Combine the children of node n into `slot` of n.
__device__ __forceinline__ void combine_body(Ctx& c, int n, int sl, int sr, int slot, bool do_ss, bool do_states) {
  const DModel& m = *c.m;
  const int16_t* ssl = node_ss(c, 2 * n, sl);
  const int16_t* ssr = node_ss(c, 2 * n + 1, sr);
  int16_t* ss = node_ss(c, n, slot);
  for (int s = c.lane; do_ss && s < m.nss; s += 32) {
    int a = ssl[s];
    ss[s] = a < 0 ? (int16_t)-1 : ssr[a];
  }
  if (do_states && c.mono) {
    const double* lwl = node_lw(c, 2 * n, sl);
    const uint16_t* tgl = node_tg(c, 2 * n, sl);
    const double* lwr = node_lw(c, 2 * n + 1, sr);
    const uint16_t* tgr = node_tg(c, 2 * n + 1, sr);
    double* lw = node_lw(c, n, slot);
    uint16_t* tg = node_tg(c, n, slot);
    for (int s = c.lane; s < m.ns; s += 32) {
      uint16_t a = tgl[s];
      int mid = a & 0x7fff;
      if (mid == 0x7fff) {
        tg[s] = 0x7fff;
        lw[s] = -DHUGE;
        continue;
      }
      uint16_t b = tgr[mid];
      if ((b & 0x7fff) == 0x7fff) {
        tg[s] = 0x7fff;
        lw[s] = -DHUGE;
        continue;
      }
      tg[s] = (uint16_t)((b & 0x7fff) | ((a ^ b) & 0x8000));
      lw[s] = lwl[s] + lwr[mid];
    }
  }
  __syncwarp();
}

// Rebuild the leaves of a proposal and their ancestors in the inactive
// slots: superstate maps (do_ss) and/or, for monomial models, state maps
// (do_states) in one traversal; `gather` collects the leaves' operators.
__device__ NOINL void tree_propose(Ctx& c, Mod& md, bool do_ss, bool do_states, bool gather) {
  const int L = c.g->L, nb = 1 << L;
  const int nleaf = md.b2 != md.b1 ? 2 : 1;
  if (gather) gather_leaves(c, md, nleaf);
  for (int q = 0; q < nleaf; ++q) {
    int b = q ? md.b2 : md.b1;
    leaf_body(c, b, q ? md.n2 : md.n1, 1 - c.act[nb + b], do_ss, do_states, q);
  }
  int n1 = nb + md.b1, n2 = nb + md.b2;
  for (int d = L - 1; d >= 0; --d) {
    n1 >>= 1;
    n2 >>= 1;
    const int cnt = n2 != n1 ? 2 : 1;
    for (int q = 0; q < cnt; ++q) {
      int n = q ? n2 : n1;
      combine_body(c, n, node_slot(c, md, 2 * n), node_slot(c, md, 2 * n + 1), 1 - c.act[n], do_ss, do_states);
    }
  }
  if (c.lane == 0) c.h->w_nodes += 2 * (L + 1);
}
__device__ void tree_accept(Ctx& c, const Mod& md) {
  const int L = c.g->L, nb = 1 << L;
  if (c.lane == 0) {
    for (int d = L; d >= 0; --d) {
      int n1 = (nb + md.b1) >> (L - d), n2 = (nb + md.b2) >> (L - d);
      c.act[n1] ^= 1;
      if (n2 != n1) c.act[n2] ^= 1;
    }
  }
  __syncwarp();
}
// Bin starts from the current operator array.
__device__ NOINL void bstart_build(Ctx& c) {
  const int nb = 1 << c.g->L, K = c.h->K;
  for (int b = c.lane; b <= nb; b += 32) c.bstart[b] = b == nb ? K : slb(c.optau, K, bin_edge(c, b));
  __syncwarp();
}
// Operators entered (+1) or left (-1) bins ba and bb.
__device__ __forceinline__ void bstart_shift(Ctx& c, int ba, int bb, int d) {
  const int nb = 1 << c.g->L;
  for (int b = c.lane; b <= nb; b += 32) c.bstart[b] += d * ((b > ba) + (b > bb));
  __syncwarp();
}
// Position of time t in the operator array (lower bound), searched inside its bin.
__device__ __forceinline__ int op_lower_bound(Ctx& c, int bin, double t) {
  const int j0 = c.bstart[bin];
  return j0 + wlb(c.optau + j0, c.bstart[bin + 1] - j0, t, c.lane);
}

// Full build from the current operator array into slot 0.
__device__ void tree_build_all(Ctx& c) {
  const int L = c.g->L, nb = 1 << L;
  Mod md;
  md.type = 0;
  bstart_build(c);
  for (int b = 0; b < nb; ++b) {
    int n = gather_bin(c, md, b, 0);
    leaf_body(c, b, n, 0, true, true, 0);
  }
  for (int n = nb - 1; n >= 1; --n) combine_body(c, n, 0, 0, 0, true, true);
  for (int i = c.lane; i < 2 * nb; i += 32) c.act[i] = 0;
  __syncwarp();
}

// Superstate just before time t in the current configuration, starting from
// s at tau = 0.
__device__ NOINL int old_prefix(Ctx& c, int s, double t) {
  const int L = c.g->L, nb = 1 << L;
  const DModel& m = *c.m;
  int b = bin_of(c, t);
  int node = 1, lo = 0, span = nb;
  for (int d = 0; d < L && s >= 0; ++d) {
    int half = span >> 1;
    if (b >= lo + half) {
      s = node_ss(c, 2 * node, c.act[2 * node])[s];
      node = 2 * node + 1;
      lo += half;
    } else {
      node = 2 * node;
    }
    span = half;
  }
  if (s < 0) return -1;
  int j0 = c.bstart[b];
  int j1 = j0 + wlb(c.optau + j0, c.bstart[b + 1] - j0, t, c.lane);
  for (int j = j0; j < j1 && s >= 0; ++j) {
    int code = c.opcode[j];
    s = m.connect[((size_t)s * m.nf + (code >> 1)) * 2 + (code & 1)];
  }
  return s;
}
// Superstate at beta reached from superstate s just before time t through
// the proposed configuration's operators at times >= t.
// t is the later member of the proposal, so its leaf is md.b2 whose
// operators tree_propose gathered already.
__device__ NOINL int new_suffix(Ctx& c, const Mod& md, int s, double t) {
  const int L = c.g->L, nb = 1 << L;
  const DModel& m = *c.m;
  const int b = md.b2;
  const int buf = md.b2 != md.b1 ? 1 : 0;
  const int n = md.b2 != md.b1 ? md.n2 : md.n1;
  const long long tb = tkey(t);
  for (int j = 0; j < n && s >= 0; ++j) {
    if (tkey(c.btau[buf][j]) < tb) continue;
    int code = c.bcode[buf][j];
    s = m.connect[((size_t)s * m.nf + (code >> 1)) * 2 + (code & 1)];
  }
  // right siblings of the left-child nodes on the leaf-to-root path, deepest
  // (earliest in time) first
  for (int d = L; d >= 1 && s >= 0; --d) {
    int node = (nb + b) >> (L - d);
    if (node & 1) continue;
    int sib = node | 1;
    s = node_ss(c, sib, node_slot(c, md, sib))[s];
  }
  return s;
}

// Trace of superstate s0 from the root state map in `slot`:
// sum over states i of s0 mapped onto themselves of sign*exp(lw).
// lg/sg: log|trace| and its sign; mx/sum: trace = sum * exp(mx) (the
// acceptance ratio uses these without a logarithm).
__device__ NOINL void root_trace(Ctx& c, int slot, int s0, double& mx_out, double& sum_out,
                                 double ref = -DHUGE) {
  const DModel& m = *c.m;
  const double* lw = node_lw(c, 1, slot);
  const uint16_t* tg = node_tg(c, 1, slot);
  int off = m.sst_off[s0], n0 = m.sst_n[s0];
  if (ref > -DHUGE) {
    // relative to a known log scale (the current trace): one exponential
    // per state and no separate scale pass; falls back when a term could
    // overflow or all underflow
    double sum = 0.0;
    bool big = false;
    for (int i = c.lane; i < n0; i += 32) {
      const int st = off + i;
      const uint16_t t = tg[st];
      if ((t & 0x7fff) != st) continue;
      const double d = lw[st] - ref;
      if (d > 600.0) big = true;
      else sum += ((t & 0x8000) ? -1.0 : 1.0) * exp(d);
    }
    if (!__any_sync(FULL, big)) {
      sum = wsum(sum);
      if (sum != 0.0) {
        mx_out = ref;
        sum_out = sum;
        return;
      }
    }
  }
  double mx = -DHUGE;
  for (int i = c.lane; i < n0; i += 32) {
    int st = off + i;
    if ((tg[st] & 0x7fff) == st) mx = fmax(mx, lw[st]);
  }
  mx = wmax(mx);
  if (mx == -DHUGE) {
    mx_out = -DHUGE;
    sum_out = 0.0;
    return;
  }
  double sum = 0.0;
  for (int i = c.lane; i < n0; i += 32) {
    int st = off + i;
    uint16_t t = tg[st];
    if ((t & 0x7fff) == st) sum += ((t & 0x8000) ? -1.0 : 1.0) * exp(lw[st] - mx);
  }
  mx_out = mx;
  sum_out = wsum(sum);
}
__device__ __forceinline__ void trace_log(double mx, double sum, double& lg, double& sg) {
  if (mx == -DHUGE) {
    lg = -DHUGE;
    sg = 0.0;
  } else {
    lg = mx + log(fabs(sum));
    sg = sum >= 0.0 ? 1.0 : -1.0;
  }
}
// |weight ratio| = |trace_new/trace_old| * |det ratio| from the mantissa/
// exponent split of the new trace; logarithms only where the plain
// product could over- or underflow.
__device__ __forceinline__ double weight_ratio(double mx, double sum, double old_log, double absdet) {
  if (mx == -DHUGE || sum == 0.0) return 0.0;
  if (mx == old_log) {  // trace already relative to the current one
    const double w = fabs(sum) * absdet;
    if (w > 1e-290 && w < 1e290) return w;
  }
  double e = mx - old_log;
  if (e > -600.0 && e < 600.0) {
    double w = exp(e) * fabs(sum) * absdet;
    if (w > 1e-290 && w < 1e290) return w;
  }
  return exp(e + log(fabs(sum)) + log(absdet));
}

// ---------------------------------------------------------------------------
// Dense-block trace: time-ordered products of exp(-dtau (E - Egs)) and the
// c/c+ blocks in the H_loc eigenbasis (get_Trace_EB_fullmatrix,
// Trace.F90:5734-6100), evaluated for all outer states at once: every outer
// state is one column of a matrix propagated through the operators, each
// column with its own log scale (the role of split_log, Trace.F90:5341-5348).
//
// Teams.  The threads that evaluate one chain's dense-block trace together:
// one warp (the chain's own warp in the phase-synchronous and independent-
// warp sweeps, and every leader-only path) or a whole block of T warps (the
// team sweep, k_sweep_team).  Values the team shares are written by its
// thread 0 and read after a team barrier; `red` is shared scratch of one
// double per warp for team reductions.
struct Team {
  int tid, nth;
  double* red;
};
__device__ __forceinline__ Team solo_team(const Ctx& c) { return Team{c.lane, 32, nullptr}; }
__device__ __forceinline__ void tsync(const Team& t) {
  if (t.nth == 32) __syncwarp();
  else __syncthreads();
}
__device__ __forceinline__ double tsum(const Team& t, double x) {
  x = wsum(x);
  if (t.nth == 32) return x;
  if ((t.tid & 31) == 0) t.red[t.tid >> 5] = x;
  __syncthreads();
  double s = 0.0;
  for (int w = 0; w < (t.nth >> 5); ++w) s += t.red[w];
  __syncthreads();
  return s;
}
__device__ __forceinline__ double tmax(const Team& t, double x) {
  x = wmax(x);
  if (t.nth == 32) return x;
  if ((t.tid & 31) == 0) t.red[t.tid >> 5] = x;
  __syncthreads();
  double s = -DHUGE;
  for (int w = 0; w < (t.nth >> 5); ++w) s = fmax(s, t.red[w]);
  __syncthreads();
  return s;
}

struct OpIter {
  int j, K, stage;  // stage: number of inserted ops consumed
};
__device__ __forceinline__ bool next_op(const Ctx& c, const Mod& md, OpIter& it, double& t, int& code) {
  while (true) {
    while (md.type == 2 && it.j < it.K && (it.j == md.ix || it.j == md.iy)) it.j++;
    bool haveOld = it.j < it.K;
    double to = haveOld ? c.optau[it.j] : 0.0;
    if (md.type == 1 && it.stage < 2) {
      double tn = it.stage == 0 ? md.t1 : md.t2;
      if (!haveOld || tn < to) {
        t = tn;
        code = it.stage == 0 ? md.c1 : md.c2;
        it.stage++;
        return true;
      }
    }
    if (!haveOld) return false;
    t = to;
    code = c.opcode[it.j];
    it.j++;
    return true;
  }
}

// ---------------------------------------------------------------------------
// Checkpoints at the bin edges: the reference's cached kets/bras with lazy
// extension (get_Trace_EB, Trace.F90:5354-5546, and the R/L loops of
// get_Trace_EB_fullmatrix), kept at the 2^L + 1 time-bin edges.  Ket
// checkpoint j: every outer state propagated from tau = 0 through the
// operators before edge j and evolved to the edge; bra checkpoint j: from
// beta through the operators after edge j.  A pair move in bins b1 <= b2
// needs kets up to b1 and bras from b2 + 1 and recomputes only bins
// b1..b2; acceptance keeps those checkpoints.
struct ChkHead {
  int sst, rows, cols, pad;
};
__device__ __forceinline__ ChkHead* chk_head(const Ctx& c, int dir, int j) {
  return (ChkHead*)(c.g->base + (size_t)c.chain * c.g->stride + c.g->o_chk +
                    ((size_t)dir * ((1 << c.g->L) + 1) + j) * c.g->chk_bytes);
}
__device__ __forceinline__ double* chk_lg(ChkHead* p) { return (double*)(p + 1); }
__device__ __forceinline__ double* chk_v(const Ctx& c, ChkHead* p) { return chk_lg(p) + c.m->nsmax; }

// work space of the dense trace: two nsmax x nsmax matrices (0, 1) and two
// nsmax vectors (2: column logs, 3: per-row / per-column factors)
__device__ __forceinline__ double* dwork(const Ctx& c, int i) {
  const size_t n2 = (size_t)c.m->nsmax * c.m->nsmax;
  return i < 2 ? c.dense + i * n2 : c.dense + 2 * n2 + (size_t)(i - 2) * c.m->nsmax;
}
// Column-wise renormalisation: each column is scaled by the power of two at
// or below its largest magnitude (exact), whose exponent goes into the
// column's log.  One warp per column (columns strided over the team's
// warps), the maximum taken on the bit patterns (order-preserving for
// magnitudes), so no FP64 compares.
__device__ void col_split(Ctx& c, int rows, int cols, double* v, double* lg, const Team& t) {
  const int ld = c.m->nsmax, lane = t.tid & 31;
  for (int col = t.tid >> 5; col < cols; col += t.nth >> 5) {
    double* vc = v + (size_t)col * ld;
    long long mk = 0;
    for (int i = lane; i < rows; i += 32) {
      const long long k = __double_as_longlong(vc[i]) & 0x7FFFFFFFFFFFFFFFll;
      mk = k > mk ? k : mk;
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      const long long y = __shfl_xor_sync(FULL, mk, o);
      mk = y > mk ? y : mk;
    }
    const int ef = (int)(mk >> 52);  // biased exponent of the maximum
    if (mk == 0 || ef == 0 || ef == 0x7FF) continue;  // zero, subnormal or non-finite column: left as is
    const int e = ef - 1023 > 1022 ? 1022 : ef - 1023;  // keep 2^-e a normal number
    if (e == 0) continue;
    const double sc = __longlong_as_double((long long)(1023 - e) << 52);  // 2^-e
    for (int i = lane; i < rows; i += 32) vc[i] *= sc;
    if (lane == 0) lg[col] += (double)e * 0.69314718055994530942;  // e ln 2
  }
  tsync(t);
}
// exp(-(E - E0) dt) on the rows of superstate sst, E0 - Egs into the logs
__device__ void col_evolve(Ctx& c, int sst, int rows, int cols, double* v, double* lg, double dt, const Team& t) {
  const DModel& m = *c.m;
  const int ld = m.nsmax;
  const double* E = m.eval + m.sst_off[sst];
  const double e0 = E[0];
  if (rows > 1) {
    double* fac = dwork(c, 3);  // one exponential per row, shared by the columns
    for (int i = t.tid; i < rows; i += t.nth) fac[i] = exp(-(E[i] - e0) * dt);
    tsync(t);
    for (int e = t.tid; e < rows * cols; e += t.nth) {
      const int i = e % rows, col = e / rows;
      v[(size_t)col * ld + i] *= fac[i];
    }
  }
  for (int col = t.tid; col < cols; col += t.nth) lg[col] += -(e0 - m.egs) * dt;
  tsync(t);
  if (rows > 1) col_split(c, rows, cols, v, lg, t);
}

// out (nn x cols) = B^T v with B the block stored as B[r * nn + i] (rows r
// of v, rows i of out), leading dimension ld for v and out.  CUDA cores:
// each thread accumulates one output row over four columns (four
// independent FMA chains; the block element is loaded once for the four).
__device__ __forceinline__ void block_gemm_fma(const double* __restrict__ B, int nn, int rows,
                                               const double* __restrict__ v, int cols, double* __restrict__ out,
                                               int ld, const Team& t) {
  const int ncb = (cols + 3) >> 2;
  for (int e = t.tid; e < nn * ncb; e += t.nth) {
    const int i = e % nn, c0 = (e / nn) * 4;
    const double* vp = v + (size_t)c0 * ld;
    double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
    if (c0 + 4 <= cols) {
#pragma unroll 4
      for (int r = 0; r < rows; ++r) {
        const double b = B[(size_t)r * nn + i];
        a0 = fma(b, vp[r], a0);
        a1 = fma(b, vp[ld + r], a1);
        a2 = fma(b, vp[2 * ld + r], a2);
        a3 = fma(b, vp[3 * ld + r], a3);
      }
      double* op = out + (size_t)c0 * ld + i;
      op[0] = a0;
      op[ld] = a1;
      op[2 * ld] = a2;
      op[3 * ld] = a3;
    } else {
      const int nc = cols - c0;
      for (int r = 0; r < rows; ++r) {
        const double b = B[(size_t)r * nn + i];
        a0 = fma(b, vp[r], a0);
        if (nc > 1) a1 = fma(b, vp[ld + r], a1);
        if (nc > 2) a2 = fma(b, vp[2 * ld + r], a2);
      }
      double* op = out + (size_t)c0 * ld + i;
      op[0] = a0;
      if (nc > 1) op[ld] = a1;
      if (nc > 2) op[2 * ld] = a2;
    }
  }
}
// The same on the FP64 tensor cores: m8n8k4 MMAs, each warp computing an
// 8 x 16 strip of out (two 8 x 8 accumulator tiles sharing the A
// fragment) over k-steps of 4, strips strided over the team's warps.
// Fragment layouts of mma.m8n8k4.f64 (PTX ISA): A row = lane / 4, k =
// lane % 4; B k = lane % 4, column = lane / 4; C row = lane / 4, columns
// 2 (lane % 4) + {0, 1}.  Out-of-range rows, columns and k are zero.
__device__ __forceinline__ void dmma_884(double& d0, double& d1, double a, double b) {
  asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
               : "+d"(d0), "+d"(d1)
               : "d"(a), "d"(b));
}
__device__ __forceinline__ void block_gemm_mma(const double* __restrict__ B, int nn, int rows,
                                               const double* __restrict__ v, int cols, double* __restrict__ out,
                                               int ld, const Team& t) {
  const int lane = t.tid & 31, warp = t.tid >> 5, nw = t.nth >> 5;
  const int ti = (nn + 7) >> 3, tj = (cols + 15) >> 4;
  const int fr = lane >> 2, fk = lane & 3;
  for (int s = warp; s < ti * tj; s += nw) {
    const int i0 = (s % ti) * 8, j0 = (s / ti) * 16;
    const int ia = i0 + fr, jb0 = j0 + fr, jb1 = j0 + 8 + fr;
    double d0 = 0.0, d1 = 0.0, d2 = 0.0, d3 = 0.0;
    for (int k0 = 0; k0 < rows; k0 += 4) {
      const int k = k0 + fk;
      const bool kin = k < rows;
      const double a = (kin && ia < nn) ? B[(size_t)k * nn + ia] : 0.0;
      const double b0 = (kin && jb0 < cols) ? v[(size_t)jb0 * ld + k] : 0.0;
      const double b1 = (kin && jb1 < cols) ? v[(size_t)jb1 * ld + k] : 0.0;
      dmma_884(d0, d1, a, b0);
      dmma_884(d2, d3, a, b1);
    }
    const int orow = i0 + fr, oc = j0 + 2 * fk;
    if (orow < nn) {
      if (oc < cols) out[(size_t)oc * ld + orow] = d0;
      if (oc + 1 < cols) out[(size_t)(oc + 1) * ld + orow] = d1;
      if (oc + 8 < cols) out[(size_t)(oc + 8) * ld + orow] = d2;
      if (oc + 9 < cols) out[(size_t)(oc + 9) * ld + orow] = d3;
    }
  }
}

// One operator: evolve by dt in superstate *sst, apply the block of
// (code, ca-flip for bras) into `out`, split.  Returns false when the
// superstate sequence breaks.  Blocks of at least 16 x 16 go to the FP64
// tensor cores when the group asks for them (CTHYB_FLAG_DMMA).
__device__ bool col_step(Ctx& c, int& sst, int& rows, int cols, double*& v, double*& out, double* lg, int code,
                         bool bra, double dt, const Team& t) {
  const DModel& m = *c.m;
  const int ld = m.nsmax;
  const int f = code >> 1, ca = bra ? 1 - (code & 1) : (code & 1);
  const int nxt = m.connect[((size_t)sst * m.nf + f) * 2 + ca];
  if (nxt < 0) return false;
  col_evolve(c, sst, rows, cols, v, lg, dt, t);
  const int nn = m.sst_n[nxt];
  const double* B = m.blk + m.blk_off[((size_t)sst * m.nf + f) * 2 + ca];
  if (t.tid == 0) {
    c.h->w_tflops += 2ll * nn * rows * cols;
    c.h->w_tbytes += 8ll * (nn * rows + rows * cols + nn * cols);
  }
  if (c.g->dmma && nn >= 16 && rows >= 16) block_gemm_mma(B, nn, rows, v, cols, out, ld, t);
  else block_gemm_fma(B, nn, rows, v, cols, out, ld, t);
  tsync(t);
  if (nn > 1 || rows > 1) col_split(c, nn, cols, out, lg, t);
  double* tmp = v;
  v = out;
  out = tmp;
  sst = nxt;
  rows = nn;
  return true;
}
__device__ void chk_load(Ctx& c, ChkHead* h, int& sst, int& rows, int& cols, double* v, double* lg, const Team& t) {
  sst = h->sst;
  rows = h->rows;
  cols = h->cols;
  const int ld = c.m->nsmax;
  const double* src = chk_v(c, h);
  for (int e = t.tid; e < rows * cols; e += t.nth) {
    const size_t x = (size_t)(e / rows) * ld + e % rows;
    v[x] = src[x];
  }
  for (int col = t.tid; col < cols; col += t.nth) lg[col] = chk_lg(h)[col];
  tsync(t);
}
__device__ void chk_store(Ctx& c, ChkHead* h, int sst, int rows, int cols, const double* v, const double* lg,
                          const Team& t) {
  const int ld = c.m->nsmax;
  double* dst = chk_v(c, h);
  for (int e = t.tid; e < rows * cols; e += t.nth) {
    const size_t x = (size_t)(e / rows) * ld + e % rows;
    dst[x] = v[x];
  }
  for (int col = t.tid; col < cols; col += t.nth) chk_lg(h)[col] = lg[col];
  if (t.tid == 0) {
    h->sst = sst;
    h->rows = rows;
    h->cols = cols;
  }
  tsync(t);
}
__device__ void chk_identity(Ctx& c, ChkHead* h, int s0, const Team& t) {
  const int ld = c.m->nsmax, n0 = c.m->sst_n[s0];
  double* dst = chk_v(c, h);
  for (int e = t.tid; e < n0 * n0; e += t.nth) dst[(size_t)(e / n0) * ld + e % n0] = (e / n0 == e % n0) ? 1.0 : 0.0;
  for (int col = t.tid; col < n0; col += t.nth) chk_lg(h)[col] = 0.0;
  if (t.tid == 0) {
    h->sst = s0;
    h->rows = n0;
    h->cols = n0;
  }
  tsync(t);
}
// Kets valid up to edge `upto` (current configuration).
__device__ NOINL bool ensure_kets(Ctx& c, int upto, const Team& t) {
  Hdr& h = *c.h;
  if (h.kv < 0) {
    chk_identity(c, chk_head(c, 0, 0), h.outer_sst, t);
    if (t.tid == 0) h.kv = 0;
    tsync(t);
  }
  double *v = dwork(c, 0), *o = dwork(c, 1), *lg = dwork(c, 2);
  while (h.kv < upto) {
    const int j = h.kv;
    int sst, rows, cols;
    chk_load(c, chk_head(c, 0, j), sst, rows, cols, v, lg, t);
    double tt = bin_edge(c, j);
    for (int i = c.bstart[j]; i < c.bstart[j + 1]; ++i) {
      const double tau = c.optau[i];
      if (!col_step(c, sst, rows, cols, v, o, lg, c.opcode[i], false, tau - tt, t)) return false;
      tt = tau;
    }
    col_evolve(c, sst, rows, cols, v, lg, bin_edge(c, j + 1) - tt, t);
    chk_store(c, chk_head(c, 0, j + 1), sst, rows, cols, v, lg, t);
    if (t.tid == 0) h.kv = j + 1;
    tsync(t);
  }
  return true;
}
// Bras valid from edge `from` (current configuration).
__device__ NOINL bool ensure_bras(Ctx& c, int from, const Team& t) {
  Hdr& h = *c.h;
  const int nb = 1 << c.g->L;
  if (h.bv > nb) {
    chk_identity(c, chk_head(c, 1, nb), h.outer_sst, t);
    if (t.tid == 0) h.bv = nb;
    tsync(t);
  }
  double *v = dwork(c, 0), *o = dwork(c, 1), *lg = dwork(c, 2);
  while (h.bv > from) {
    const int j = h.bv;
    int sst, rows, cols;
    chk_load(c, chk_head(c, 1, j), sst, rows, cols, v, lg, t);
    double tt = bin_edge(c, j);
    for (int i = c.bstart[j] - 1; i >= c.bstart[j - 1]; --i) {
      const double tau = c.optau[i];
      if (!col_step(c, sst, rows, cols, v, o, lg, c.opcode[i], true, tt - tau, t)) return false;
      tt = tau;
    }
    col_evolve(c, sst, rows, cols, v, lg, tt - bin_edge(c, j - 1), t);
    chk_store(c, chk_head(c, 1, j - 1), sst, rows, cols, v, lg, t);
    if (t.tid == 0) h.bv = j - 1;
    tsync(t);
  }
  return true;
}
// Sum over the outer states (columns) of d[col] * exp(lg[col]) in log form
// (the sum of addLogTr, Trace.F90:298-309): log|sum| and its sign.
__device__ void col_logsum(const double* d, const double* lg, int cols, const Team& t, double& out_lg,
                           double& out_sg) {
  double mx = -DHUGE;
  for (int col = t.tid; col < cols; col += t.nth)
    if (d[col] != 0.0) mx = fmax(mx, lg[col] + log(fabs(d[col])));
  mx = tmax(t, mx);
  out_lg = -DHUGE;
  out_sg = 0.0;
  if (mx == -DHUGE) return;
  double s = 0.0;
  for (int col = t.tid; col < cols; col += t.nth)
    if (d[col] != 0.0) s += (d[col] > 0.0 ? 1.0 : -1.0) * exp(lg[col] + log(fabs(d[col])) - mx);
  s = tsum(t, s);
  if (s == 0.0) return;
  out_lg = mx + log(fabs(s));
  out_sg = s > 0.0 ? 1.0 : -1.0;
}
// <bra|ket> per column at one edge, summed over the outer states in log form.
__device__ void chk_close(Ctx& c, int sst, int rows, int cols, const double* v, double* lg, ChkHead* bh,
                          double& out_lg, double& out_sg, const Team& t) {
  out_lg = -DHUGE;
  out_sg = 0.0;
  if (bh->sst != sst) return;
  const int ld = c.m->nsmax, lane = t.tid & 31;
  const double* bv = chk_v(c, bh);
  const double* blg = chk_lg(bh);
  double* d = dwork(c, 3);  // per-column <bra|ket>
  for (int col = t.tid >> 5; col < cols; col += t.nth >> 5) {
    double part = 0.0;
    for (int i = lane; i < rows; i += 32) part = fma(v[(size_t)col * ld + i], bv[(size_t)col * ld + i], part);
    part = wsum(part);
    if (lane == 0) d[col] = part;
  }
  tsync(t);
  // column logs of ket and bra together (lg is the trace's work vector,
  // free to update here)
  for (int col = t.tid; col < cols; col += t.nth) lg[col] += blg[col];
  tsync(t);
  col_logsum(d, lg, cols, t, out_lg, out_sg);
}
// Trace of a proposed pair move for the current outer superstate from the
// checkpoints: kets at edge b1, the proposed operators of bins b1..b2 (the
// gathered leaves for b1/b2, the current lists in between), bras at b2 + 1.
__device__ NOINL void chk_trace(Ctx& c, const Mod& md, double& out_lg, double& out_sg, const Team& t) {
  out_lg = -DHUGE;
  out_sg = 0.0;
  const int b1 = md.b1, b2 = md.b2;
  if (!ensure_kets(c, b1, t) || !ensure_bras(c, b2 + 1, t)) {
    if (t.tid < 32) set_status(c, ST_INTERNAL);
    return;
  }
  double *v = dwork(c, 0), *o = dwork(c, 1), *lg = dwork(c, 2);
  int sst, rows, cols;
  chk_load(c, chk_head(c, 0, b1), sst, rows, cols, v, lg, t);
  double tt = bin_edge(c, b1);
  for (int b = b1; b <= b2; ++b) {
    const bool gathered = b == b1 || b == b2;
    const int buf = b == b1 ? 0 : 1;
    const int n = !gathered ? c.bstart[b + 1] - c.bstart[b] : (buf == 0 ? md.n1 : md.n2);
    for (int q = 0; q < n; ++q) {
      const double tau = gathered ? c.btau[buf][q] : c.optau[c.bstart[b] + q];
      const int code = gathered ? c.bcode[buf][q] : c.opcode[c.bstart[b] + q];
      if (!col_step(c, sst, rows, cols, v, o, lg, code, false, tau - tt, t)) return;
      tt = tau;
    }
    col_evolve(c, sst, rows, cols, v, lg, bin_edge(c, b + 1) - tt, t);
    tt = bin_edge(c, b + 1);
  }
  chk_close(c, sst, rows, cols, v, lg, chk_head(c, 1, b2 + 1), out_lg, out_sg, t);
}
__device__ __forceinline__ void chk_invalidate(Ctx& c) {
  if (c.lane == 0) {
    c.h->kv = -1;
    c.h->bv = (1 << c.g->L) + 1;
  }
  __syncwarp();
}
// After an accepted pair move in bins md.b1..md.b2: checkpoints outside the
// changed bins stay valid unless the outer superstate changed.
__device__ __forceinline__ void chk_keep(Ctx& c, const Mod& md, int new_outer) {
  if (!c.g->o_chk) return;
  if (new_outer != c.h->outer_sst) {
    chk_invalidate(c);
    return;
  }
  if (c.lane == 0) {
    if (c.h->kv > md.b1) c.h->kv = md.b1;
    if (c.h->bv < md.b2 + 1) c.h->bv = md.b2 + 1;
  }
  __syncwarp();
}

// Dense-block trace from scratch for outer superstate s0 over the whole
// proposed configuration: the identity for the outer states propagated from
// tau = 0 through every operator and evolved to beta; the trace is the sum
// of the diagonal elements with their column scales.  log|trace| and sign.
__device__ NOINL void dense_trace(Ctx& c, const Mod& md, int s0, double& lg, double& sg, const Team& t) {
  const int ld = c.m->nsmax, n0 = c.m->sst_n[s0];
  double *v = dwork(c, 0), *o = dwork(c, 1), *lgc = dwork(c, 2);
  for (int e = t.tid; e < n0 * n0; e += t.nth) v[(size_t)(e / n0) * ld + e % n0] = (e / n0 == e % n0) ? 1.0 : 0.0;
  for (int col = t.tid; col < n0; col += t.nth) lgc[col] = 0.0;
  tsync(t);
  lg = -DHUGE;
  sg = 0.0;
  int sst = s0, rows = n0;
  double tprev = 0.0, tau;
  int code;
  OpIter it{0, c.h->K, 0};
  while (next_op(c, md, it, tau, code)) {
    if (!col_step(c, sst, rows, n0, v, o, lgc, code, false, tau - tprev, t)) return;
    tprev = tau;
  }
  if (sst != s0) return;
  col_evolve(c, sst, rows, n0, v, lgc, c.g->beta - tprev, t);
  double* d = dwork(c, 3);
  for (int col = t.tid; col < n0; col += t.nth) d[col] = v[(size_t)col * ld + col];
  tsync(t);
  col_logsum(d, lgc, n0, t, lg, sg);
}

// ---------------------------------------------------------------------------
// Shifts of the sorted arrays

// insert value/slot at position p of a sorted array with n entries
__device__ NOINL void arr_insert(Ctx& c, double* a, short* sl, int n, int p, double v, short s) {
  for (int base = n - 1; base >= p; base -= 32) {
    int i = base - c.lane;
    bool on = i >= p;
    double x = 0;
    short y = 0;
    if (on) {
      x = a[i];
      y = sl[i];
    }
    __syncwarp();
    if (on) {
      a[i + 1] = x;
      sl[i + 1] = y;
    }
    __syncwarp();
  }
  if (c.lane == 0) {
    a[p] = v;
    sl[p] = s;
  }
  __syncwarp();
}
__device__ NOINL void arr_remove(Ctx& c, double* a, short* sl, int n, int p) {
  for (int base = p + 1; base < n; base += 32) {
    int i = base + c.lane;
    bool on = i < n;
    double x = 0;
    short y = 0;
    if (on) {
      x = a[i];
      y = sl[i];
    }
    __syncwarp();
    if (on) {
      a[i - 1] = x;
      sl[i - 1] = y;
    }
    __syncwarp();
  }
}
// global operator array: insert t1 (before old index p1) and t2 (before old
// index p2, p2 >= p1)
__device__ NOINL void ops_insert2(Ctx& c, int p1, int p2, double t1, int c1, double t2, int c2) {
  int K = c.h->K;
  for (int base = K - 1; base >= p1; base -= 32) {
    int i = base - c.lane;
    bool on = i >= p1;
    double x = 0;
    int y = 0;
    if (on) {
      x = c.optau[i];
      y = c.opcode[i];
    }
    __syncwarp();
    if (on) {
      int d = i + (i >= p2 ? 2 : 1);
      c.optau[d] = x;
      c.opcode[d] = y;
    }
    __syncwarp();
  }
  if (c.lane == 0) {
    c.optau[p1] = t1;
    c.opcode[p1] = c1;
    c.optau[p2 + 1] = t2;
    c.opcode[p2 + 1] = c2;
  }
  __syncwarp();
}
__device__ NOINL void ops_remove2(Ctx& c, int ix, int iy) {
  int K = c.h->K;
  for (int base = ix + 1; base < K; base += 32) {
    int i = base + c.lane;
    bool on = i < K && i != iy;
    double x = 0;
    int y = 0;
    if (on) {
      x = c.optau[i];
      y = c.opcode[i];
    }
    __syncwarp();
    if (on) {
      int d = i - (i > iy ? 2 : 1);
      c.optau[d] = x;
      c.opcode[d] = y;
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------
// Proposal log record
__device__ NOINL void write_record(Ctx& c, const cthyb_record& r) {
  __syncwarp();
  if (c.log && c.lane == 0) {
    Hdr& h = *c.h;
    if (h.logn < c.g->logcap) c.log[h.logn] = r;
    h.logn++;
  }
  __syncwarp();
}

// Trace of the proposed configuration for outer superstate s0.
// Trace of the proposed configuration as sum * exp(mx).
__device__ void proposed_trace(Ctx& c, Mod& md, int s0, double& mx, double& sum, const Team& t) {
  if (c.mono) {
    root_trace(c, 1 - c.act[1], s0, mx, sum, c.h->trace_log);  // state tree rebuilt after the QN check
  } else if (s0 == c.h->outer_sst && c.g->o_chk) {
    chk_trace(c, md, mx, sum, t);  // log|trace| and its sign from the checkpoints
  } else {
    dense_trace(c, md, s0, mx, sum, t);  // new outer superstate: from scratch
  }
}

// ---------------------------------------------------------------------------
// One proposal in phases.  StepAdd (CTQMC.F90:3353-3613) and StepRem
// (CTQMC.F90:3892-4151) for diagonal hybridisation, split so that a block of
// warps can execute each phase together (k_sweep_sync): draw, set-up,
// superstate/state tree + QN check, determinant ratio, trace + Metropolis
// decision, accepted-move updates, bookkeeping.  A warp whose proposal ended
// early (equal times, no pairs, QN violation, rejection) idles in the later
// phases.  The per-warp proposal state lives in shared memory.
struct Prop {
  int move, alive, rare, co, f, k, K, fpos_c, fpos_a, p1, p2, snew, np, ix, iy, cax, rank_c, rank_a, slot_c,
      slot_a, accept;
  double tau_c, tau_a, tdf, hprf, ratio, det_sign, det_log, tr_log, tr_sign, tr_mx, tr_sum, tx, ty;
  Mod md;
};

__device__ __forceinline__ void prop_end(Ctx& c, Prop& p, int outcome) {
  c.rec->outcome = outcome;
  p.alive = 0;
  __syncwarp();
}

// Phase 0: capacity check and the move-type draws (CTQMC.F90:8435-8476).
__device__ NOINL void ph_draw(Ctx& c, Prop& p) {
  Hdr& h = *c.h;
  p.alive = 0;
  p.rare = 0;
  p.accept = 0;
  for (int f = 0; f < c.m->nf; ++f)
    if (h.k[f] + 1 > c.kcap) {
      set_status(c, ST_CAPACITY);
      return;
    }
  if (h.K + 2 > c.g->opcap) {
    set_status(c, ST_CAPACITY);
    return;
  }
  // move thresholds of the Z-space loop (PercentageWormInsert = 0)
  const double rn = grnd(c);
  const double pair = __dsub_rn(__dsub_rn(1.0, c.g->p_shift), c.g->p_global);
  int move;
  if (rn < __ddiv_rn(pair, 2.0)) move = 0;
  else if (rn <= pair) move = 1;
  else if (rn <= __dsub_rn(1.0, c.g->p_shift)) move = 2;
  else move = 3;
  cthyb_record& r = *c.rec;
  for (int i = c.lane; i < (int)(sizeof(cthyb_record) / 4); i += 32) ((int*)&r)[i] = 0;
  __syncwarp();
  p.move = move;
  r.move = move;
  r.outer_sst = h.outer_sst;
  r.k_total = h.K;
  if (move >= 2) {  // global or tau-shift move
    p.rare = 1;
    __syncwarp();
    return;
  }
  if (!(grnd(c) >= c.g->p_4op)) {  // 4-operator move (StepAdd4 / StepRem4), no outer draw
    p.move = move + 5;
    r.move = move + 5;
    p.rare = 1;
    __syncwarp();
    return;
  }
  p.rare = 0;
  bool co = grnd(c) < c.g->p_outer;
  p.co = co;
  r.change_outer = co;
  if (c.lane == 0) {
    if (move == 0) h.try_add++;
    else h.try_rem++;
  }
  if (c.g->offdiag) {  // off-diagonal pair moves run in the rare-move phase
    p.move = move + 7;
    p.rare = 1;
    __syncwarp();
    return;
  }
  p.alive = 1;
  __syncwarp();
}

// Phase 1, insertion: pair_OperAdd (Trace.F90:3657-3702) and
// process_OperAdd's equal-time rejection and FPos (Trace.F90:4275-4500).
__device__ NOINL void ph_setup_add(Ctx& c, Prop& p) {
  Hdr& h = *c.h;
  const DModel& m = *c.m;
  cthyb_record& r = *c.rec;
  double u1 = grnd(c);
  int orb = randint(c, 1, m.nd);
  int spin = randint(c, 1, 2);
  double u2 = grnd(c);
  double wmin = h.tauwin_min, wmax = h.tauwin_max, tdm = h.taudiff_max;
  double tau_width = __dsub_rn(wmax, wmin);
  double tau_a = __dadd_rn(wmin, __dmul_rn(tau_width, u1));
  double tdf = __dmul_rn(1.0, tau_width);
  double tau_min = fmax(__dsub_rn(tau_a, tdm), wmin);
  double tau_w2 = __dsub_rn(fmin(__dadd_rn(tau_a, tdm), wmax), tau_min);
  double tau_c = __dadd_rn(tau_min, __dmul_rn(tau_w2, u2));
  tdf = __dmul_rn(tdf, tau_w2);
  const int f = 2 * (orb - 1) + (spin - 1);
  const int k = h.k[f];
  const int K = h.K;
  r.orb = orb;
  r.spin = spin;
  r.tau_c = tau_c;
  r.tau_a = tau_a;
  const int ba = bin_of(c, tau_a), bc = bin_of(c, tau_c);
  int pa = op_lower_bound(c, ba, tau_a);
  int pc = op_lower_bound(c, bc, tau_c);
  bool eq = teq(tau_a, tau_c) || (pa < K && teq(c.optau[pa], tau_a)) || (pc < K && teq(c.optau[pc], tau_c));
  if (eq) {
    if (c.lane == 0) h.qn_add++;
    prop_end(c, p, 0);
    return;
  }
  int fpos_c = wlb(srt_ptr(c, f, 0), k, tau_c, c.lane) + 1;
  int fpos_a = wlb(srt_ptr(c, f, 1), k, tau_a, c.lane) + 1;
  r.fpos_c = fpos_c;
  r.fpos_a = fpos_a;
  bool a_first = tau_a < tau_c;
  Mod& md = p.md;
  md.type = 1;
  md.t1 = a_first ? tau_a : tau_c;
  md.c1 = a_first ? 2 * f + 1 : 2 * f;
  md.t2 = a_first ? tau_c : tau_a;
  md.c2 = a_first ? 2 * f : 2 * f + 1;
  md.ix = md.iy = -1;
  md.b1 = a_first ? ba : bc;
  md.b2 = a_first ? bc : ba;
  p.p1 = a_first ? pa : pc;
  p.p2 = a_first ? pc : pa;
  md.p1 = p.p1;
  md.p2 = p.p2;
  p.f = f;
  p.k = k;
  p.K = K;
  p.fpos_c = fpos_c;
  p.fpos_a = fpos_a;
  p.tau_c = tau_c;
  p.tau_a = tau_a;
  p.tdf = tdf;
  __syncwarp();
}

// Phase 1, removal: gen_OperRemove (Trace.F90:4851-4960): the NPair-th
// eligible pair in (time of the earlier member, time of the later member)
// order, FPos, and the proposal-probability factor.
__device__ NOINL void ph_setup_rem(Ctx& c, Prop& p) {
  Hdr& h = *c.h;
  cthyb_record& r = *c.rec;
  if (h.npairs == -1) {
    int np = count_npairs(c);
    if (c.lane == 0) h.npairs = np;
    __syncwarp();
  }
  if (h.npairs <= 0) {
    if (c.lane == 0) h.qn_rem++;
    prop_end(c, p, 2);
    return;
  }
  const int K = h.K;
  const double wmin = h.tauwin_min, wmax = h.tauwin_max, tdm = h.taudiff_max;
  int target = randint(c, 1, h.npairs);
  int start = wlb(c.optau, K, wmin, c.lane);
  int ix = -1, yrank = -1;
  for (int base = start; base < K; base += 32) {
    int i = base + c.lane;
    int cnt = 0, lb = 0;
    if (i < K) {
      double t = c.optau[i];
      int cd = c.opcode[i], ff = cd >> 1, cc = cd & 1;
      const double* opp = srt_ptr(c, ff, 1 - cc);
      double hi = fmin(wmax, __dadd_rn(t, tdm));
      lb = sub(opp, h.k[ff], t);
      int ub = sub(opp, h.k[ff], hi);
      cnt = ub > lb ? ub - lb : 0;
    }
    int cum = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(FULL, cum, o);
      if (c.lane >= o) cum += y;
    }
    int total = __shfl_sync(FULL, cum, 31);
    if (target <= total) {
      unsigned bal = __ballot_sync(FULL, cum >= target);
      int L0 = __ffs(bal) - 1;
      int before = __shfl_sync(FULL, cum - cnt, L0);
      ix = base + L0;
      yrank = __shfl_sync(FULL, lb, L0) + (target - before) - 1;
      break;
    }
    target -= total;
  }
  if (ix < 0) {
    set_status(c, ST_INTERNAL);
    p.alive = 0;
    return;
  }
  const double tx = c.optau[ix];
  const int cx = c.opcode[ix], f = cx >> 1, cax = cx & 1;
  const int k = h.k[f];
  if (yrank < 0 || yrank >= k) {
    set_status(c, ST_INTERNAL);
    p.alive = 0;
    return;
  }
  const double ty = srt_ptr(c, f, 1 - cax)[yrank];
  const int by = bin_of(c, ty);
  const int iy = op_lower_bound(c, by, ty);
  const int xrank = wlb(srt_ptr(c, f, cax), k, tx, c.lane);
  if (iy <= ix || iy >= K || !teq(c.optau[iy], ty) || xrank >= k || !teq(srt_ptr(c, f, cax)[xrank], tx)) {
    set_status(c, ST_INTERNAL);
    p.alive = 0;
    return;
  }
  const double tau_c = cax == 0 ? tx : ty, tau_a = cax == 0 ? ty : tx;
  const int rank_c = cax == 0 ? xrank : yrank, rank_a = cax == 0 ? yrank : xrank;
  p.hprf = __ddiv_rn((double)h.npairs,
                     __dmul_rn(__dsub_rn(wmax, wmin),
                               __dsub_rn(fmin(__dadd_rn(tau_a, tdm), wmax), fmax(__dsub_rn(tau_a, tdm), wmin))));
  r.orb = f / 2 + 1;
  r.spin = f % 2 + 1;
  r.tau_c = tau_c;
  r.tau_a = tau_a;
  r.fpos_c = rank_c + 1;
  r.fpos_a = rank_a + 1;
  r.npairs = h.npairs;
  Mod& md = p.md;
  md.type = 2;
  md.ix = ix;
  md.iy = iy;
  md.t1 = tx;
  md.t2 = ty;
  md.c1 = md.c2 = 0;
  md.b1 = bin_of(c, tx);
  md.b2 = by;
  p.f = f;
  p.k = k;
  p.K = K;
  p.ix = ix;
  p.iy = iy;
  p.cax = cax;
  p.tx = tx;
  p.ty = ty;
  p.tau_c = tau_c;
  p.tau_a = tau_a;
  p.rank_c = rank_c;
  p.rank_a = rank_a;
  p.fpos_c = rank_c + 1;
  p.fpos_a = rank_a + 1;
  p.slot_c = sslot_ptr(c, f, 0)[rank_c];
  p.slot_a = sslot_ptr(c, f, 1)[rank_a];
  __syncwarp();
}

// Phase 2: proposed tree and the quantum-number check
// (check_sst_sequence, Trace.F90:1243-1304; CTQMC.F90:3421-3470 and
// 3928-3976).
__device__ NOINL void ph_tree_ss(Ctx& c, Prop& p) {
  Hdr& h = *c.h;
  Mod& md = p.md;
  tree_propose(c, md, true, false, true);  // superstate maps (integer only)
  int root_new = 1 - c.act[1];
  int s0 = h.outer_sst, snew = s0;
  bool ok;
  if (!p.co) {
    ok = node_ss(c, 1, root_new)[s0] == s0;
  } else {
    int inside = old_prefix(c, s0, md.t2);
    snew = inside >= 0 ? new_suffix(c, md, inside, md.t2) : -1;
    ok = snew >= 0 && node_ss(c, 1, root_new)[snew] == snew;
  }
  p.snew = snew;
  __syncwarp();
  if (!ok) {
    if (c.lane == 0) {
      if (p.move == 0) h.qn_add++;
      else h.qn_rem++;
    }
    prop_end(c, p, 1);
  }
}

// Phase 2b: state maps and log weights of the proposed tree (monomial
// models), only for proposals that passed the QN check.
__device__ NOINL void ph_tree_states(Ctx& c, Prop& p) {
  if (c.mono) tree_propose(c, p.md, false, true, false);
}

// Phase 3: determinant ratio.  Insertion: S - R.(M Q)
// (get_LogDetRatPairAdd / get_DetRatAdd, Trace.F90:2775-2833,
// MatrixUpdate.F90:392-407); removal: M(c, a) (Trace.F90:2937-2966).
__device__ NOINL void ph_det(Ctx& c, Prop& p) {
  Hdr& h = *c.h;
  const int f = p.f, k = p.k;
  const double* Mf = M_ptr(c, f);
  if (p.move == 1) {
    double dr = Mf[(size_t)p.slot_a * c.kcap + p.slot_c];
    double sig = ((p.fpos_c - p.fpos_a) & 1) ? -1.0 : 1.0;
    p.ratio = dr;
    p.det_sign = (dr >= 0.0 ? 1.0 : -1.0) * sig;
    __syncwarp();
    return;
  }
  double* Q = c.scr;
  double* R = c.scr + c.kcap;
  double* v = c.scr + 2 * c.kcap;
  const double* tcs = stau_ptr(c, f, 0);
  const double* tas = stau_ptr(c, f, 1);
  const double tau_c = p.tau_c, tau_a = p.tau_a;
  for (int i = c.lane; i < k; i += 32) {
    Q[i] = hybrf(c, __dsub_rn(tas[i], tau_c), f);
    R[i] = hybrf(c, __dsub_rn(tau_a, tcs[i]), f);
  }
  double S = hybrf(c, __dsub_rn(tau_a, tau_c), f);
  __syncwarp();
  double part = 0.0;
  for (int i = c.lane; i < k; i += 32) {
    double acc = 0.0;
    for (int j = 0; j < k; ++j) acc = fma(Mf[(size_t)j * c.kcap + i], Q[j], acc);
    v[i] = acc;
    part = fma(R[i], acc, part);
  }
  double ratio = S - wsum(part);
  double sig = ((p.fpos_c - p.fpos_a) & 1) ? -1.0 : 1.0;
  p.ratio = ratio;
  p.det_sign = (ratio >= 0.0 ? 1.0 : -1.0) * sig;
  if (c.lane == 0) {
    h.w_mbytes += 8ll * k * k + 32ll * k;
    h.w_mflops += 2ll * k * k + 2ll * k;
  }
  __syncwarp();
}

// Phase 4: trace of the proposed configuration, NPairs of the new
// configuration (update_NPairs / ensure_valid_NPairs, Trace.F90:1756-1922)
// and the Metropolis decision (CTQMC.F90:3508-3524, 4050-4058).
__device__ NOINL void ph_trace(Ctx& c, Prop& p) {
  double tr_mx, tr_sum;
  proposed_trace(c, p.md, p.snew, tr_mx, tr_sum, solo_team(c));
  p.tr_mx = tr_mx;
  p.tr_sum = tr_sum;
  __syncwarp();
}
// The same evaluated by a team of warps (dense-block models in the team
// sweep; monomial traces stay with the chain's own warp, thread 0's warp).
__device__ NOINL void ph_trace_team(Ctx& c, Prop& p, const Team& t) {
  if (c.mono) {
    if (t.tid < 32) ph_trace(c, p);
    __syncthreads();
    return;
  }
  double tr_mx, tr_sum;
  proposed_trace(c, p.md, p.snew, tr_mx, tr_sum, t);
  if (t.tid == 0) {
    p.tr_mx = tr_mx;
    p.tr_sum = tr_sum;
  }
  __syncthreads();
}
__device__ NOINL void ph_decide(Ctx& c, Prop& p) {
  Hdr& h = *c.h;
  const DModel& m = *c.m;
  cthyb_record& r = *c.rec;
  const double tr_mx = p.tr_mx, tr_sum = p.tr_sum;
  const double wmin = h.tauwin_min, wmax = h.tauwin_max, tdm = h.taudiff_max;
  const int f = p.f, k = p.k, K = p.K;
  double prob, rnd;
  if (p.move == 0) {
    const Mod& md = p.md;
    rnd = grnd(c);
    int np;
    if (h.npairs == -1) {
      // full recount including the new pair
      int tot = 0;
      int start = wlb(c.optau, K, wmin, c.lane);
      for (int i = start + c.lane; i < K; i += 32) {
        double t = c.optau[i];
        if (t > wmax) continue;
        int cd = c.opcode[i], ff = cd >> 1, cc = cd & 1;
        int n = cnt_later(srt_ptr(c, ff, 1 - cc), h.k[ff], t, wmax, tdm);
        if (ff == f) {
          double tn = cc == 0 ? p.tau_a : p.tau_c;  // partner among the new operators
          if (tn > t && tn <= fmin(wmax, __dadd_rn(t, tdm))) n++;
        }
        tot += n;
      }
      tot = wsumi(tot);
      int n = 0;
      if (c.lane == 0) {
        if (md.t1 >= wmin && md.t1 <= wmax) {  // pairs with a new operator as the earlier member
          n += cnt_later(srt_ptr(c, f, 1 - (md.c1 & 1)), k, md.t1, wmax, tdm);
          if (md.t2 <= fmin(wmax, __dadd_rn(md.t1, tdm))) n += 1;
        }
        if (md.t2 >= wmin && md.t2 <= wmax) n += cnt_later(srt_ptr(c, f, 1 - (md.c2 & 1)), k, md.t2, wmax, tdm);
      }
      np = tot + __shfl_sync(FULL, n, 0);
    } else {
      int n = partner_counts(c, srt_ptr(c, f, 1 - (md.c1 & 1)), k, md.t1, srt_ptr(c, f, 1 - (md.c2 & 1)), k, md.t2,
                             wmin, wmax, tdm);
      if (md.t2 <= wmax && md.t2 <= __dadd_rn(md.t1, tdm)) n += 1;
      np = h.npairs + n;
    }
    double wr = weight_ratio(tr_mx, tr_sum, h.trace_log, fabs(p.ratio));
    prob = fabs(p.tdf * (double)(2 * m.nd) / (double)np * wr);
    p.np = np;
    r.npairs = np;
  } else {
    double wr = weight_ratio(tr_mx, tr_sum, h.trace_log, fabs(p.ratio));
    prob = fabs(p.hprf / (double)(2 * m.nd) * wr);
    rnd = grnd(c);
  }
  bool accept = rnd < prob;
  if (accept && p.move == 1 && fabs(p.ratio) < 1e-12) {  // CTQMC.F90:4062
    set_status(c, ST_NUMERIC);
    p.alive = 0;
    return;
  }
  double det_log = 0.0, tr_lg = 0.0, tr_sg = 0.0;
  if (accept || c.log) {
    det_log = log(fabs(p.ratio));
    trace_log(tr_mx, tr_sum, tr_lg, tr_sg);
  }
  r.det_log = det_log;
  r.det_sign = p.det_sign;
  r.tr_log = tr_lg;
  r.tr_sign = tr_sg;
  r.prob = prob;
  r.rand = rnd;
  p.det_log = det_log;
  p.tr_log = tr_lg;
  p.tr_sign = tr_sg;
  p.accept = accept;
  __syncwarp();
  if (!accept) prop_end(c, p, 3);
}

// AccPair (CTQMC.F90:3579-3582, 4112-4122): an accepted pair insertion or
// removal of flavour f whose operators are dt apart, binned as
// min(Ntau, floor(dt / beta * Ntau) + 1) (NAccPair = NGtau, AccPairMax =
// beta in the warmup and measurement loops, CTQMC.F90:8203-8204).
__device__ __forceinline__ void count_accpair(const Ctx& c, int f, double dt) {
  if (!c.g->o_accpair || c.lane != 0) return;
  const int nt = c.g->ntau;
  int bin = (int)floor(__dmul_rn(__ddiv_rn(dt, c.g->beta), (double)nt)) + 1;
  bin = bin > nt ? nt : (bin < 1 ? 1 : bin);
  ((double*)(c.g->base + (size_t)c.chain * c.g->stride + c.g->o_accpair))[(size_t)f * nt + bin - 1] += 1.0;
}

// Phase 5: accepted insertion: get_MatAdd in slot order (w = R^T M, rank-one
// update, new row and column), sorted and operator arrays, tree flip, sign.
__device__ NOINL void ph_accept_add(Ctx& c, Prop& p) {
  Hdr& h = *c.h;
  const int f = p.f, k = p.k, K = p.K;
  const Mod& md = p.md;
  const double* R = c.scr + c.kcap;
  const double* v = c.scr + 2 * c.kcap;
  double* w = c.scr + 3 * c.kcap;
  double* Mw = M_ptr(c, f);
  for (int j = c.lane; j < k; j += 32) {
    double acc = 0.0;
    const double* col = Mw + (size_t)j * c.kcap;
    for (int i = 0; i < k; ++i) acc = fma(R[i], col[i], acc);
    w[j] = acc;
  }
  __syncwarp();
  double invS = 1.0 / p.ratio;
  for (int i = c.lane; i < k; i += 32) {
    double vi = v[i] * invS;
    for (int j = 0; j < k; ++j) Mw[(size_t)j * c.kcap + i] = fma(vi, w[j], Mw[(size_t)j * c.kcap + i]);
    Mw[(size_t)k * c.kcap + i] = -vi;
  }
  for (int j = c.lane; j < k; j += 32) Mw[(size_t)j * c.kcap + k] = -w[j] * invS;
  if (c.lane == 0) {
    Mw[(size_t)k * c.kcap + k] = invS;
    h.w_mbytes += 16ll * k * k + 16ll * k;
    h.w_mflops += 4ll * k * k;
    stau_ptr(c, f, 0)[k] = p.tau_c;
    stau_ptr(c, f, 1)[k] = p.tau_a;
  }
  __syncwarp();
  arr_insert(c, srt_ptr(c, f, 0), sslot_ptr(c, f, 0), k, p.fpos_c - 1, p.tau_c, (short)k);
  arr_insert(c, srt_ptr(c, f, 1), sslot_ptr(c, f, 1), k, p.fpos_a - 1, p.tau_a, (short)k);
  ops_insert2(c, p.p1, p.p2, md.t1, md.c1, md.t2, md.c2);
  bstart_shift(c, md.b1, md.b2, +1);
  tree_accept(c, md);
  chk_keep(c, md, p.snew);
  if (c.lane == 0) {
    h.k[f] = k + 1;
    h.K = K + 2;
    h.det_log = p.det_log + h.det_log;
    h.det_sign = p.det_sign * h.det_sign;
    h.trace_log = p.tr_log;
    h.trace_sign = p.tr_sign;
    h.npairs = p.np;
    h.outer_sst = p.snew;
    h.acc_add++;
    h.acc_since_refresh++;
    h.w_opbytes += 24ll * (K - p.p1) + 40ll * k;
    count_accpair(c, f, __dsub_rn(md.t2, md.t1));
  }
  __syncwarp();
  double sgn = config_sign(c);
  if (c.lane == 0) h.cfgsign = -sgn;
  c.rec->outcome = 4;
  __syncwarp();
}

// Phase 5: accepted removal: get_MatRem in slot order, then the last row and
// column move into the gap; arrays, tree flip, NPairs, sign.
__device__ NOINL void ph_accept_rem(Ctx& c, Prop& p) {
  Hdr& h = *c.h;
  const int f = p.f, k = p.k, K = p.K, slot_c = p.slot_c, slot_a = p.slot_a;
  const Mod& md = p.md;
  double* Mw = M_ptr(c, f);
  double* col = c.scr;           // column slot_a
  double* row = c.scr + c.kcap;  // row slot_c
  for (int i = c.lane; i < k; i += 32) {
    col[i] = Mw[(size_t)slot_a * c.kcap + i];
    row[i] = Mw[(size_t)i * c.kcap + slot_c];
  }
  __syncwarp();
  double inv = 1.0 / p.ratio;
  for (int i = c.lane; i < k; i += 32) {
    double ci = col[i] * inv;
    for (int j = 0; j < k; ++j) Mw[(size_t)j * c.kcap + i] = fma(-ci, row[j], Mw[(size_t)j * c.kcap + i]);
  }
  __syncwarp();
  const int last = k - 1;
  if (slot_c != last)
    for (int j = c.lane; j < k; j += 32) Mw[(size_t)j * c.kcap + slot_c] = Mw[(size_t)j * c.kcap + last];
  __syncwarp();
  if (slot_a != last)
    for (int i = c.lane; i < k; i += 32) Mw[(size_t)slot_a * c.kcap + i] = Mw[(size_t)last * c.kcap + i];
  __syncwarp();
  if (c.lane == 0) {
    h.w_mbytes += 16ll * k * k;
    h.w_mflops += 2ll * k * k;
  }
  arr_remove(c, srt_ptr(c, f, 0), sslot_ptr(c, f, 0), k, p.rank_c);
  arr_remove(c, srt_ptr(c, f, 1), sslot_ptr(c, f, 1), k, p.rank_a);
  if (slot_c != last) {
    short* ss = sslot_ptr(c, f, 0);
    for (int i = c.lane; i < k - 1; i += 32)
      if (ss[i] == last) ss[i] = (short)slot_c;
    if (c.lane == 0) stau_ptr(c, f, 0)[slot_c] = stau_ptr(c, f, 0)[last];
  }
  if (slot_a != last) {
    short* ss = sslot_ptr(c, f, 1);
    for (int i = c.lane; i < k - 1; i += 32)
      if (ss[i] == last) ss[i] = (short)slot_a;
    if (c.lane == 0) stau_ptr(c, f, 1)[slot_a] = stau_ptr(c, f, 1)[last];
  }
  __syncwarp();
  ops_remove2(c, p.ix, p.iy);
  bstart_shift(c, md.b1, md.b2, -1);
  tree_accept(c, md);
  chk_keep(c, md, p.snew);
  const double wmin = h.tauwin_min, wmax = h.tauwin_max, tdm = h.taudiff_max;
  // update_NPairs(-1): the pair and the partners of its members
  const int gone = 1 + partner_counts(c, srt_ptr(c, f, 1 - p.cax), k - 1, p.tx, srt_ptr(c, f, p.cax), k - 1, p.ty,
                                      wmin, wmax, tdm);
  if (c.lane == 0) {
    h.k[f] = k - 1;
    h.K = K - 2;
    h.det_log = p.det_log + h.det_log;
    h.det_sign = p.det_sign * h.det_sign;
    h.trace_log = p.tr_log;
    h.trace_sign = p.tr_sign;
    h.outer_sst = p.snew;
    h.acc_rem++;
    h.acc_since_refresh++;
    count_accpair(c, f, __dsub_rn(p.ty, p.tx));
    h.w_opbytes += 24ll * (K - p.ix) + 40ll * k;
    h.npairs -= gone;
  }
  __syncwarp();
  double sgn = config_sign(c);
  if (c.lane == 0) h.cfgsign = -sgn;
  c.rec->outcome = 4;
  __syncwarp();
}

// Phase 6: record, proposal count and the window cadence
// (CTQMC.F90:8531: shift every NSlide add/remove tries).
__device__ NOINL void ph_finish(Ctx& c, Prop& p) {
  Hdr& h = *c.h;
  cthyb_record& r = *c.rec;
  r.outer_sst = h.outer_sst;
  r.k_total = h.K;
  __syncwarp();
  write_record(c, r);
  if (c.lane == 0) h.nprop++;
  __syncwarp();
  // after every move, whatever its kind (CTQMC.F90:8531-8533)
  if ((h.try_add + h.try_rem) % h.nslide == 0) shift_window(c);
}

// ---------------------------------------------------------------------------
// Global and tau-shift moves.  Rare (PercentageGlobalMove and
// PercentageTauShiftMove default to 0.5 % each); each rebuilds the whole
// tree into the inactive node slots, so a rejection leaves the active tree
// untouched and an acceptance flips every node.  Work space per chain
// (o_glob): the new inverse matrices, the new sorted time lists, a copy of
// the operator arrays.
__device__ __forceinline__ double* glob_minv(const Ctx& c) {
  return (double*)(c.g->base + (size_t)c.chain * c.g->stride + c.g->o_glob);
}
__device__ __forceinline__ double* glob_srt(const Ctx& c) {
  return glob_minv(c) + (size_t)c.m->nf * c.kcap * c.kcap;
}
__device__ __forceinline__ double* glob_optau(const Ctx& c) { return glob_srt(c) + (size_t)c.m->nf * 2 * c.kcap; }
__device__ __forceinline__ int* glob_opcode(const Ctx& c) { return (int*)(glob_optau(c) + c.g->opcap + 2); }

__device__ NOINL void tree_build_inactive(Ctx& c, bool do_ss, bool do_states) {
  const int L = c.g->L, nb = 1 << L;
  Mod md;
  md.type = 0;
  for (int b = 0; b < nb; ++b) {
    const int n = gather_bin(c, md, b, 0);
    leaf_body(c, b, n, 1 - c.act[nb + b], do_ss, do_states, 0);
  }
  for (int n = nb - 1; n >= 1; --n)
    combine_body(c, n, 1 - c.act[2 * n], 1 - c.act[2 * n + 1], 1 - c.act[n], do_ss, do_states);
  if (c.lane == 0) c.h->w_nodes += 2 * nb;
}
__device__ __forceinline__ void tree_flip_all(Ctx& c) {
  for (int i = c.lane; i < (2 << c.g->L); i += 32) c.act[i] ^= 1;
  __syncwarp();
}

// Running product of pivot magnitudes kept as a mantissa in [1, 2) and a
// binary exponent: one FP64 multiply per pivot and one logarithm per matrix
// instead of a logarithm per pivot (each costs tens of dependent FP64
// operations).  A product that would leave the normal range falls back to
// adding log(x) directly.
__device__ __forceinline__ void pivot_mul(double& m, long long& e, double& dlog, double x) {
  const double y = m * x;
  const long long b = __double_as_longlong(y);
  const int ef = (int)((b >> 52) & 0x7FF);
  if (ef == 0 || ef == 0x7FF) {
    dlog += log(x);
    return;
  }
  e += ef - 1023;
  m = __longlong_as_double((b & 0x000FFFFFFFFFFFFFll) | 0x3FF0000000000000ll);
}
__device__ __forceinline__ double pivot_log(double m, long long e) {
  return log(m) + (double)e * 0.69314718055994530942;
}

// Gauss-Jordan inverse with partial pivoting (first maximal pivot) of the
// k x k matrix H (column-major, leading dimension kcap) into I, which must
// hold the identity on entry; log|det| and sign accumulate into dlog/dsign.
// False for a singular matrix.
__device__ NOINL bool gj_eliminate(Ctx& c, int k, double* H, double* I, double& dlog, double& dsign) {
  const int ld = c.kcap;
  double pm = 1.0;
  long long pe = 0;
  for (int j = 0; j < k; ++j) {
    double best = -1.0;
    int bi = j;
    for (int i = j + c.lane; i < k; i += 32) {
      const double a = fabs(H[(size_t)j * ld + i]);
      if (a > best) {
        best = a;
        bi = i;
      }
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      const double ob = __shfl_xor_sync(FULL, best, o);
      const int oi = __shfl_xor_sync(FULL, bi, o);
      if (ob > best || (ob == best && oi < bi)) {
        best = ob;
        bi = oi;
      }
    }
    if (best <= 0.0) return false;
    if (bi != j) {
      for (int col = c.lane; col < k; col += 32) {
        double t = H[(size_t)col * ld + j];
        H[(size_t)col * ld + j] = H[(size_t)col * ld + bi];
        H[(size_t)col * ld + bi] = t;
        t = I[(size_t)col * ld + j];
        I[(size_t)col * ld + j] = I[(size_t)col * ld + bi];
        I[(size_t)col * ld + bi] = t;
      }
      dsign = -dsign;
    }
    __syncwarp();
    const double piv = H[(size_t)j * ld + j];
    pivot_mul(pm, pe, dlog, fabs(piv));
    if (piv < 0) dsign = -dsign;
    const double ip = 1.0 / piv;
    for (int col = c.lane; col < k; col += 32) {
      H[(size_t)col * ld + j] *= ip;
      I[(size_t)col * ld + j] *= ip;
    }
    __syncwarp();
    // rank-one elimination of every (row i, column col) outside row and
    // column j, the lanes over all k x k elements at once (column j and row
    // j are only read here)
    for (int e = c.lane; e < k * k; e += 32) {
      const int i = e % k, col = e / k;
      if (i == j || col == j) continue;
      const double fct = H[(size_t)j * ld + i];
      H[(size_t)col * ld + i] -= fct * H[(size_t)col * ld + j];
      I[(size_t)col * ld + i] -= fct * I[(size_t)col * ld + j];
    }
    __syncwarp();
    for (int i = c.lane; i < k; i += 32)
      if (i != j) {
        I[(size_t)j * ld + i] -= H[(size_t)j * ld + i] * I[(size_t)j * ld + j];
        H[(size_t)j * ld + i] = 0.0;
      }
    __syncwarp();
  }
  dlog += pivot_log(pm, pe);
  return true;
}

// Gauss-Jordan inverse of H(a_rank, c_rank) = Delta(tau_a - tau_c) for the
// sorted time lists sc/sa of flavour f (get_InvFullHybr, Trace.F90:2279-2336);
// log|det| and sign are accumulated into dlog/dsign (get_MatLogDetFull,
// MatrixUpdate.F90:41-99).  On return work + kcap^2 holds the inverse,
// element (c_rank, a_rank) at [a_rank * kcap + c_rank].  Returns false for a
// singular matrix.
__device__ NOINL bool gj_inverse(Ctx& c, int f, int k, const double* sc, const double* sa, double* work,
                                 double& dlog, double& dsign) {
  const int ld = c.kcap;
  double* H = work;
  double* I = work + (size_t)ld * ld;
  for (int e = c.lane; e < k * k; e += 32) {
    int ia = e % k, ic = e / k;
    H[(size_t)ic * ld + ia] = hybrf(c, __dsub_rn(sa[ia], sc[ic]), f);
    I[(size_t)ic * ld + ia] = (ia == ic) ? 1.0 : 0.0;
  }
  __syncwarp();
  return gj_eliminate(c, k, H, I, dlog, dsign);
}

// log|det| and sign of the current inverse matrix of flavour f in rank order
// by LU with partial pivoting (first maximal pivot), accumulated into
// dlog/dsign (get_FullLogDet, Trace.F90:2665-2685, via get_LogDetFull).
__device__ NOINL void lu_logdet_minv(Ctx& c, int f, double* work, double& dlog, double& dsign) {
  const int k = c.h->k[f], ld = c.kcap;
  if (k == 0) return;
  const short* slc = sslot_ptr(c, f, 0);
  const short* sla = sslot_ptr(c, f, 1);
  const double* Mf = M_ptr(c, f);
  double* A = work;  // A(rc, ra) at [ra * ld + rc]
  for (int e = c.lane; e < k * k; e += 32) {
    const int rc = e % k, ra = e / k;
    A[(size_t)ra * ld + rc] = Mf[(size_t)sla[ra] * ld + slc[rc]];
  }
  __syncwarp();
  double pm = 1.0;
  long long pe = 0;
  for (int j = 0; j < k; ++j) {
    double best = -1.0;
    int bi = j;
    for (int i = j + c.lane; i < k; i += 32) {
      const double a = fabs(A[(size_t)j * ld + i]);
      if (a > best) {
        best = a;
        bi = i;
      }
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      const double ob = __shfl_xor_sync(FULL, best, o);
      const int oi = __shfl_xor_sync(FULL, bi, o);
      if (ob > best || (ob == best && oi < bi)) {
        best = ob;
        bi = oi;
      }
    }
    if (best <= 0.0) {
      dlog = -DHUGE;
      dsign = 0.0;
      return;
    }
    if (bi != j) {
      for (int col = c.lane; col < k; col += 32) {
        const double t = A[(size_t)col * ld + j];
        A[(size_t)col * ld + j] = A[(size_t)col * ld + bi];
        A[(size_t)col * ld + bi] = t;
      }
      dsign = -dsign;
    }
    __syncwarp();
    const double piv = A[(size_t)j * ld + j];
    pivot_mul(pm, pe, dlog, fabs(piv));
    if (piv < 0) dsign = -dsign;
    for (int i = j + 1 + c.lane; i < k; i += 32) A[(size_t)j * ld + i] /= piv;
    __syncwarp();
    const int r = k - j - 1;  // trailing block, the lanes over all its r x r elements
    for (int e = c.lane; e < r * r; e += 32) {
      const int i = j + 1 + e % r, col = j + 1 + e / r;
      A[(size_t)col * ld + i] -= A[(size_t)j * ld + i] * A[(size_t)col * ld + j];
    }
    __syncwarp();
  }
  dlog += pivot_log(pm, pe);
}

// Per-flavour sorted time lists of the current operator arrays into
// dst[(2f + ca) * kcap + rank]; counts into k (lane-uniform).
__device__ NOINL void sorted_lists(Ctx& c, double* dst, int* k) {
  const int K = c.h->K;
  for (int f = 0; f < c.m->nf; ++f)
    for (int ca = 0; ca < 2; ++ca) {
      double* st = dst + (size_t)(2 * f + ca) * c.kcap;
      int n = 0;
      for (int base = 0; base < K; base += 32) {
        const int i = base + c.lane;
        const bool is = i < K && c.opcode[i] == 2 * f + ca;
        const unsigned bal = __ballot_sync(FULL, is);
        const int pos = n + __popc(bal & ((1u << c.lane) - 1u));
        if (is && pos < c.kcap) st[pos] = c.optau[i];
        n += __popc(bal);
      }
      if (ca == 0) k[f] = n;
    }
  __syncwarp();
}

// Trace of the configuration in the operator arrays with outer superstate
// s0, from the inactive tree slots (monomial models: state maps rebuilt
// there first) or the dense product.
__device__ NOINL void rebuilt_trace(Ctx& c, int s0, double& lg, double& sg) {
  if (c.mono) {
    tree_build_inactive(c, false, true);
    double mx, sum;
    root_trace(c, 1 - c.act[1], s0, mx, sum);
    trace_log(mx, sum, lg, sg);
  } else {
    Mod md;
    md.type = 0;
    dense_trace(c, md, s0, lg, sg, solo_team(c));
  }
}

// off-diagonal branches of the global and tau-shift moves (defined with the
// off-diagonal pair moves below)
__device__ NOINL void global_od_tail(Ctx& c, int K, int new_outer, double factor, const int* opc_old);
__device__ NOINL double shift_od_rotate(Ctx& c, const double* tau_old, const int* opc_old, int K, double dtau);
__device__ NOINL double od_cfgsign(Ctx& c);

// StepGlob, CTQMC.F90:4433-4554: spin flip (30 %, gen_SpinFlipUpdate),
// creator/annihilator flip (30 %, gen_CAFlip), a user symmetry move or its
// inverse (20 % when NSymMove > 0, gen_SymUpdate), otherwise a random
// flavour permutation with random CA flip (gen_GlobalUpdate_new,
// rand_perm) (Trace.F90:1083-1198); QN checks perform_spinflip_check_qn /
// perform_global_check_qn (Trace.F90:1306-1394); full inverse and
// determinant (get_InvFullHybr) times the LU determinant of the current
// inverse matrices (get_FullLogDet); weight exp(dlog tr + log detrat) * sst
// factor.
__device__ NOINL void ph_global(Ctx& c, Prop& p) {
  Hdr& h = *c.h;
  const DModel& m = *c.m;
  cthyb_record& r = *c.rec;
  if (c.lane == 0) h.try_glob++;
  __syncwarp();
  const int K = h.K, nd = m.nd, n2 = 2 * nd;
  if (K == 0) {
    r.outcome = 2;
    __syncwarp();
    return;
  }
  int gu[NFMAX + 1];
  int type;
  const double u = grnd(c);
  if (u < 0.3) {
    type = 3;  // spin flip
    gu[0] = 0;
    for (int i = 1; i <= n2; ++i) gu[i] = i <= nd ? i + nd : i - nd;
  } else if (u < 0.6) {
    type = 4;  // CA flip
    gu[0] = 1;
    for (int i = 1; i <= n2; ++i) gu[i] = i;
  } else if (u < 0.8 && c.g->nsym > 0) {
    type = 2;  // user symmetry move or its inverse (gen_SymUpdate)
    const int isym = randint(c, 1, 2 * c.g->nsym);
    gu[0] = 0;
    for (int i = 1; i <= n2; ++i) gu[i] = c.g->symmoves[(size_t)(isym - 1) * n2 + (i - 1)];
  } else {
    type = 1;  // random permutation (Green 1963) and random CA flip
    for (int i = 1; i <= n2; ++i) gu[i] = i;
    for (int j = 1; j <= n2; ++j) {
      const int i = randint(c, j, n2);
      const int t = gu[j];
      gu[j] = gu[i];
      gu[i] = t;
    }
    gu[0] = randint(c, 0, 1);
  }
  // flavour f = 2b + s -> reference index b + Nd*s + 1 -> gu -> new flavour
  int fmap[NFMAX];
  for (int f = 0; f < m.nf; ++f) {
    const int g = gu[(f >> 1) + nd * (f & 1) + 1] - 1;
    fmap[f] = 2 * (g % nd) + g / nd;
  }
  const int flip = gu[0] != 0;
  int* opc_old = glob_opcode(c);
  for (int i = c.lane; i < K; i += 32) {
    const int code = c.opcode[i];
    opc_old[i] = code;
    c.opcode[i] = 2 * fmap[code >> 1] + (flip ? 1 - (code & 1) : (code & 1));
  }
  __syncwarp();
  // QN check on the superstate maps of the rebuilt tree
  tree_build_inactive(c, true, false);
  const int16_t* ss_new = node_ss(c, 1, 1 - c.act[1]);
  const int16_t* ss_old = node_ss(c, 1, c.act[1]);
  int new_outer = h.outer_sst;
  double factor;
  if (type == 3 && m.has_szt) {
    new_outer = m.sflip_sst[h.outer_sst];
    factor = ss_new[new_outer] == new_outer ? 1.0 : 0.0;
  } else {
    int n_old = 0, n_new = 0;
    for (int s = c.lane; s < m.nss; s += 32) {
      n_old += ss_old[s] == s;
      n_new += ss_new[s] == s;
    }
    n_old = wsumi(n_old);
    n_new = wsumi(n_new);
    if (n_old <= 0) {
      set_status(c, ST_INTERNAL);  // "impossible old configuration"
      return;
    }
    if (n_new <= 0) {
      factor = 0.0;
    } else {
      factor = __ddiv_rn((double)n_new, (double)n_old);
      int kk = randint(c, 1, n_new);
      if (c.lane == 0)
        for (int s = 0; s < m.nss; ++s)
          if (ss_new[s] == s && --kk <= 0) {
            new_outer = s;
            break;
          }
      new_outer = __shfl_sync(FULL, new_outer, 0);
    }
  }
  r.orb = type;
  r.spin = gu[0];
  r.fpos_c = new_outer;
  r.tau_c = factor;
  if (factor == 0.0) {
    for (int i = c.lane; i < K; i += 32) c.opcode[i] = opc_old[i];
    if (c.lane == 0) h.qn_glob++;
    r.outcome = 1;
    __syncwarp();
    return;
  }
  if (c.g->offdiag) {  // one inverse matrix over all flavours
    global_od_tail(c, K, new_outer, factor, opc_old);
    return;
  }
  // new sorted lists and inverse matrices
  double* srt_new = glob_srt(c);
  double* minv_new = glob_minv(c);
  int knew[NFMAX];
  sorted_lists(c, srt_new, knew);
  double dlog = 0.0, dsign = 1.0;
  bool singular = false;
  for (int f = 0; f < m.nf && !singular; ++f) {
    const int k = knew[f];
    if (k == 0) continue;
    const double* sc = srt_new + (size_t)(2 * f) * c.kcap;
    if (!gj_inverse(c, f, k, sc, sc + c.kcap, c.dense, dlog, dsign)) {
      singular = true;
      break;
    }
    const double* I = c.dense + (size_t)c.kcap * c.kcap;
    double* Mf = minv_new + (size_t)f * c.kcap * c.kcap;
    for (int e = c.lane; e < k * k; e += 32) {
      const int rc = e % k, ra = e / k;
      Mf[(size_t)ra * c.kcap + rc] = I[(size_t)ra * c.kcap + rc];
    }
    __syncwarp();
  }
  // DetRat = DetNew * det(current inverse matrices)
  double olog = 0.0, osign = 1.0;
  if (!singular)
    for (int f = 0; f < m.nf; ++f) lu_logdet_minv(c, f, c.dense, olog, osign);
  double tr_lg = -DHUGE, tr_sg = 0.0, prob = 0.0;
  const double det_lg = singular ? -DHUGE : dlog + olog;
  const double det_sg = singular ? 0.0 : dsign * osign;
  if (!singular) {
    rebuilt_trace(c, new_outer, tr_lg, tr_sg);
    prob = fabs(exp(__dsub_rn(tr_lg, h.trace_log) + det_lg) * factor);
  }
  const double rnd = grnd(c);
  r.det_log = det_lg;
  r.det_sign = det_sg;
  r.tr_log = tr_lg;
  r.tr_sign = tr_sg;
  r.prob = prob;
  r.rand = rnd;
  if (rnd < prob) {
    for (int f = 0; f < m.nf; ++f) {
      const int k = knew[f];
      const double* src = minv_new + (size_t)f * c.kcap * c.kcap;
      double* Mf = M_ptr(c, f);
      for (int e = c.lane; e < k * k; e += 32) {
        const size_t idx = (size_t)(e / k) * c.kcap + (e % k);
        Mf[idx] = src[idx];
      }
      for (int ca = 0; ca < 2; ++ca) {
        const double* st = srt_new + (size_t)(2 * f + ca) * c.kcap;
        for (int i = c.lane; i < k; i += 32) {
          srt_ptr(c, f, ca)[i] = st[i];
          sslot_ptr(c, f, ca)[i] = (short)i;
          stau_ptr(c, f, ca)[i] = st[i];
        }
      }
    }
    __syncwarp();
    tree_flip_all(c);
    if (c.g->o_chk) chk_invalidate(c);
    if (c.lane == 0) {
      for (int f = 0; f < m.nf; ++f) h.k[f] = knew[f];
      h.det_log = dlog;
      h.det_sign = dsign;
      h.trace_log = tr_lg;
      h.trace_sign = tr_sg;
      h.outer_sst = new_outer;
      h.acc_glob++;
    }
    __syncwarp();
    const double sgn = config_sign(c);
    if (c.lane == 0) h.cfgsign = -sgn;
    r.outcome = 4;
  } else {
    for (int i = c.lane; i < K; i += 32) c.opcode[i] = opc_old[i];
    r.outcome = 3;
  }
  __syncwarp();
}

// StepChangeOuter, CTQMC.F90:4570-4638 (no state sampling): new outer
// superstate in proportion to the normalised empty-trace weights; always
// accepted.
__device__ NOINL void ph_change_outer(Ctx& c, Prop& p) {
  Hdr& h = *c.h;
  cthyb_record& r = *c.rec;
  r.move = 4;
  double lg = -DHUGE, sg = 0.0;
  int s0 = h.outer_sst;
  for (int tries = 0; tries < 64 && !(lg > -DHUGE); ++tries) {
    const double rnd = grnd(c);
    r.rand = rnd;
    if (c.lane == 0) {
      double acc = 0.0;
      for (int s = 0; s < c.m->nss; ++s) {
        s0 = s;
        acc += c.g->empty_w[s];
        if (acc >= rnd && c.g->empty_w[s] != 0.0) break;
      }
    }
    s0 = __shfl_sync(FULL, s0, 0);
    if (c.mono) {
      double mx, sum;
      root_trace(c, c.act[1], s0, mx, sum);
      trace_log(mx, sum, lg, sg);
    } else {
      Mod md;
      md.type = 0;
      dense_trace(c, md, s0, lg, sg, solo_team(c));
    }
  }
  if (!(lg > -DHUGE)) {
    set_status(c, ST_INTERNAL);
    return;
  }
  if (c.lane == 0) {
    h.outer_sst = s0;
    h.trace_log = lg;
    h.trace_sign = sg;
  }
  __syncwarp();
  if (c.g->o_chk) chk_invalidate(c);
  const double sgn = config_sign(c);
  if (c.lane == 0) h.cfgsign = -sgn;
  r.outcome = 4;
  r.tr_log = lg;
  r.tr_sign = sg;
  __syncwarp();
}

// StepShiftTau_proper, CTQMC.F90:4641-4835, and
// update_InvFullHybrShiftTau_diag (Trace.F90:2355-2452): every time moves by
// -DeltaTau cyclically; the operators that wrap go to the end of the list;
// the outer superstate becomes the one entering the new first operator; the
// window keeps its place relative to the operators.  On acceptance M keeps
// its entries (slot order), negated where exactly one of the creator and
// the annihilator wrapped, and the determinant sign flips for an odd
// dimension with an odd number of wrapped rows and columns.
__device__ NOINL void ph_shift(Ctx& c, Prop& p) {
  Hdr& h = *c.h;
  const DModel& m = *c.m;
  cthyb_record& r = *c.rec;
  const int K = h.K;
  if (K == 0) {
    ph_change_outer(c, p);
    return;
  }
  const double beta = c.g->beta;
  const double dtau = __dmul_rn(grnd(c), beta);
  r.tau_c = dtau;
  if (dtau == 0.0 || dtau == beta) {
    r.outcome = 2;
    __syncwarp();
    return;
  }
  if (c.lane == 0) h.try_shift++;
  __syncwarp();
  const int first = wlb(c.optau, K, dtau, c.lane);  // first operator with tau >= DeltaTau
  const int new_outer = first < K ? old_prefix(c, h.outer_sst, dtau) : h.outer_sst;
  double* tau_old = glob_optau(c);
  int* opc_old = glob_opcode(c);
  for (int i = c.lane; i < K; i += 32) {
    tau_old[i] = c.optau[i];
    opc_old[i] = c.opcode[i];
  }
  __syncwarp();
  for (int i = c.lane; i < K; i += 32) {
    const int j = i + first < K ? i + first : i + first - K;
    const double x = __dsub_rn(tau_old[j], dtau);  // modulo(tau - DeltaTau, beta)
    c.optau[i] = x < 0.0 ? __dadd_rn(x, beta) : x;
    c.opcode[i] = opc_old[j];
  }
  __syncwarp();
  bstart_build(c);
  const int wp_old = h.window_position, np_old = h.npairs;
  const double wmin_old = h.tauwin_min, wmax_old = h.tauwin_max;
  {
    const int nw = h.num_windows;
    const int d = (int)floor(__dmul_rn(__ddiv_rn(dtau, beta), (double)(nw + 1)));
    const int dm = ((d % nw) + nw) % nw;
    if (c.lane == 0) {
      h.window_position = (((wp_old - dm) % nw) + nw) % nw;
      h.npairs = -1;
    }
    __syncwarp();
    set_window_bounds(c);
  }
  tree_build_inactive(c, true, false);
  double tr_lg, tr_sg;
  rebuilt_trace(c, new_outer, tr_lg, tr_sg);
  const double prob = fabs(exp(__dsub_rn(tr_lg, h.trace_log)));
  const double rnd = grnd(c);
  r.fpos_c = new_outer;
  r.tr_log = tr_lg;
  r.tr_sign = tr_sg;
  r.prob = prob;
  r.rand = rnd;
  if (rnd < prob) {
    double detrat = 1.0;
    double* tmp = glob_srt(c);
    short* tmps = (short*)glob_minv(c);
    if (c.g->offdiag) detrat = shift_od_rotate(c, tau_old, opc_old, K, dtau);
    for (int f = 0; f < m.nf && !c.g->offdiag; ++f) {
      const int k = h.k[f];
      if (k == 0) continue;
      const double* tc = stau_ptr(c, f, 0);
      const double* ta = stau_ptr(c, f, 1);
      double* Mf = M_ptr(c, f);
      for (int e = c.lane; e < k * k; e += 32) {
        const int sc = e % k, sa = e / k;
        if ((tc[sc] < dtau) != (ta[sa] < dtau)) Mf[(size_t)sa * c.kcap + sc] = -Mf[(size_t)sa * c.kcap + sc];
      }
      int w[2];
      for (int ca = 0; ca < 2; ++ca) {
        double* st = srt_ptr(c, f, ca);
        short* sl = sslot_ptr(c, f, ca);
        double* sv = stau_ptr(c, f, ca);
        w[ca] = wlb(st, k, dtau, c.lane);
        for (int i = c.lane; i < k; i += 32) {
          const int j = i + w[ca] < k ? i + w[ca] : i + w[ca] - k;
          const double x = __dsub_rn(st[j], dtau);
          tmp[i] = x < 0.0 ? __dadd_rn(x, beta) : x;
          tmps[i] = sl[j];
        }
        __syncwarp();
        for (int i = c.lane; i < k; i += 32) {
          st[i] = tmp[i];
          sl[i] = tmps[i];
          const double x = __dsub_rn(sv[i], dtau);
          sv[i] = x < 0.0 ? __dadd_rn(x, beta) : x;
        }
        __syncwarp();
      }
      if ((k & 1) && ((w[0] + w[1]) & 1)) detrat = -detrat;
    }
    tree_flip_all(c);
    if (c.g->o_chk) chk_invalidate(c);
    if (c.lane == 0) {
      h.trace_log = tr_lg;
      h.trace_sign = tr_sg;
      h.outer_sst = new_outer;
      h.det_sign = h.det_sign * detrat;
      h.acc_shift++;
    }
    __syncwarp();
    const double cs = c.g->offdiag ? od_cfgsign(c) : -config_sign(c);
    if (c.lane == 0) h.cfgsign = cs;
    r.outcome = 4;
  } else {
    for (int i = c.lane; i < K; i += 32) {
      c.optau[i] = tau_old[i];
      c.opcode[i] = opc_old[i];
    }
    __syncwarp();
    bstart_build(c);
    if (c.lane == 0) {
      h.window_position = wp_old;
      h.tauwin_min = wmin_old;
      h.tauwin_max = wmax_old;
      h.npairs = np_old;
    }
    r.outcome = 3;
  }
  __syncwarp();
}

// ---------------------------------------------------------------------------
// 4-operator moves (StepAdd4 / StepRem4, CTQMC.F90:3615-3890, 4153-4431),
// diagonal hybridisation.  Rare like global moves: the proposed operator
// arrays are written in place (the old ones saved in the o_glob work space),
// the changed flavours' inverse matrices are rebuilt by Gauss-Jordan and the
// tree into the inactive slots; a rejection restores the arrays.  The
// reference rebuilds every flavour's matrix; for the unchanged flavours the
// ratio of the rebuilt and the present determinant is one, so only the
// changed flavours enter here.

// Removable pairs of the operator arrays (time order, K entries) without the
// entries skip[0..3] (-1: unused) (ensure_valid_NPairs_diag,
// Trace.F90:1762-1803, on the list without them).
// A creator/annihilator pair of codes cx, cy: opposite kinds, and the same
// flavour unless the hybridisation is off-diagonal (is_rempair_diag /
// is_rempair_offdiag, Trace.F90:1994-2030).
__device__ __forceinline__ bool pair_codes(const Ctx& c, int cx, int cy) {
  return ((cx & 1) != (cy & 1)) && (c.g->offdiag || (cx >> 1) == (cy >> 1));
}
__device__ NOINL int count_pairs_skip(Ctx& c, const double* tau, const int* code, int K, const int* skip) {
  const Hdr& h = *c.h;
  const double wmin = h.tauwin_min, wmax = h.tauwin_max, tdm = h.taudiff_max;
  int tot = 0;
  for (int i = c.lane; i < K; i += 32) {
    if (i == skip[0] || i == skip[1] || i == skip[2] || i == skip[3]) continue;
    const double x = tau[i];
    if (x < wmin || x > wmax) continue;
    const int cx = code[i];
    const double hi = fmin(wmax, __dadd_rn(x, tdm));
    for (int j = i + 1; j < K; ++j) {
      if (tau[j] > hi) break;
      if (j == skip[0] || j == skip[1] || j == skip[2] || j == skip[3]) continue;
      const int cy = code[j];
      tot += pair_codes(c, cx, cy);
    }
  }
  return wsumi(tot);
}

// The target-th removable pair (1-based) in the scan order of
// gen_OperRemove (Trace.F90:4880-4910) without the skip entries: indices
// ix < iy, lane-uniform; false if there is none.
__device__ NOINL bool select_pair_skip(Ctx& c, const double* tau, const int* code, int K, const int* skip,
                                       int target, int& ix, int& iy) {
  const Hdr& h = *c.h;
  const double wmin = h.tauwin_min, wmax = h.tauwin_max, tdm = h.taudiff_max;
  const int start = wlb(tau, K, wmin, c.lane);
  for (int base = start; base < K; base += 32) {
    const int i = base + c.lane;
    int cnt = 0;
    if (i < K && i != skip[0] && i != skip[1] && i != skip[2] && i != skip[3]) {
      const double x = tau[i];
      const int cx = code[i];
      const double hi = fmin(wmax, __dadd_rn(x, tdm));
      for (int j = i + 1; j < K; ++j) {
        if (tau[j] > hi) break;
        if (j == skip[0] || j == skip[1] || j == skip[2] || j == skip[3]) continue;
        const int cy = code[j];
        cnt += pair_codes(c, cx, cy);
      }
    }
    int cum = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(FULL, cum, o);
      if (c.lane >= o) cum += y;
    }
    const int total = __shfl_sync(FULL, cum, 31);
    if (target <= total) {
      const unsigned bal = __ballot_sync(FULL, cum >= target);
      const int L0 = __ffs(bal) - 1;
      const int before = __shfl_sync(FULL, cum - cnt, L0);
      int want = target - before, jy = -1;
      if (c.lane == L0) {
        const double x = tau[i];
        const int cx = code[i];
        const double hi = fmin(wmax, __dadd_rn(x, tdm));
        for (int j = i + 1; j < K; ++j) {
          if (tau[j] > hi) break;
          if (j == skip[0] || j == skip[1] || j == skip[2] || j == skip[3]) continue;
          const int cy = code[j];
          if (pair_codes(c, cx, cy) && --want <= 0) {
            jy = j;
            break;
          }
        }
      }
      ix = base + L0;
      iy = __shfl_sync(FULL, jy, L0);
      return iy > ix;
    }
    target -= total;
  }
  return false;
}

// is_rempair (Trace.F90:1994-2030) for (time, code) operators.
__device__ __forceinline__ bool rempair4(const Ctx& c, const Hdr& h, double tx, int cx, double ty, int cy) {
  return pair_codes(c, cx, cy) && tx >= h.tauwin_min && tx <= h.tauwin_max &&
         ty >= h.tauwin_min && ty <= h.tauwin_max && fabs(__dsub_rn(tx, ty)) <= h.taudiff_max;
}

// hybpairremfactor of gen_OperRemove (Trace.F90:4942-4948); ta is the
// annihilator's time.
__device__ __forceinline__ double remfac4(const Hdr& h, int np, double ta) {
  return __ddiv_rn((double)np, __dmul_rn(__dsub_rn(h.tauwin_max, h.tauwin_min),
                                         __dsub_rn(fmin(__dadd_rn(ta, h.taudiff_max), h.tauwin_max),
                                                   fmax(__dsub_rn(ta, h.taudiff_max), h.tauwin_min))));
}

// Superstate walk over operators j0 .. j1-1 of the present arrays, skipping
// the entries in skip[0..3], from superstate s (lane 0 walks; lane-uniform).
__device__ NOINL int walk_ops(Ctx& c, int s, int j0, int j1, const int* skip) {
  const DModel& m = *c.m;
  if (c.lane == 0)
    for (int j = j0; j < j1 && s >= 0; ++j) {
      if (j == skip[0] || j == skip[1] || j == skip[2] || j == skip[3]) continue;
      const int code = c.opcode[j];
      s = m.connect[((size_t)s * m.nf + (code >> 1)) * 2 + (code & 1)];
    }
  return __shfl_sync(FULL, s, 0);
}

// Determinant ratio of the proposed arrays for the changed flavours fa, fb
// (new sorted lists in srt_new, counts in knew, new inverses in the o_glob
// matrices), the trace from the rebuilt tree, the Metropolis draw and the
// installation on acceptance.  `factor` multiplies the weight ratio; the
// old arrays are in glob_optau/glob_opcode (K_old entries).  Returns the
// outcome (3 rejected, 4 accepted).
__device__ NOINL int rebuild4_decide(Ctx& c, int fa, int fb, double factor, int K_old, int np_new) {
  Hdr& h = *c.h;
  cthyb_record& r = *c.rec;
  double* srt_new = glob_srt(c);
  double* minv_new = glob_minv(c);
  int knew[NFMAX];
  bstart_build(c);
  tree_build_inactive(c, true, false);
  sorted_lists(c, srt_new, knew);
  double dlog = 0.0, dsign = 1.0, olog = 0.0, osign = 1.0;
  bool singular = false;
  for (int q = 0; q < 2 && !singular; ++q) {
    const int f = q == 0 ? fa : fb;
    if (q == 1 && fb == fa) break;
    const int k = knew[f];
    if (k > 0) {
      const double* sc = srt_new + (size_t)(2 * f) * c.kcap;
      if (!gj_inverse(c, f, k, sc, sc + c.kcap, c.dense, dlog, dsign)) {
        singular = true;
        break;
      }
      const double* I = c.dense + (size_t)c.kcap * c.kcap;
      double* Mf = minv_new + (size_t)f * c.kcap * c.kcap;
      for (int e = c.lane; e < k * k; e += 32) {
        const int rc = e % k, ra = e / k;
        Mf[(size_t)ra * c.kcap + rc] = I[(size_t)ra * c.kcap + rc];
      }
      __syncwarp();
    }
    lu_logdet_minv(c, f, c.dense, olog, osign);
  }
  double tr_lg = -DHUGE, tr_sg = 0.0, prob = 0.0;
  const double det_lg = singular ? -DHUGE : dlog + olog;
  const double det_sg = singular ? 0.0 : dsign * osign;
  if (!singular) {
    rebuilt_trace(c, h.outer_sst, tr_lg, tr_sg);
    prob = fabs(__dmul_rn(factor, exp(__dsub_rn(tr_lg, h.trace_log) + det_lg)));
  }
  const double rnd = grnd(c);
  r.det_log = det_lg;
  r.det_sign = det_sg;
  r.tr_log = tr_lg;
  r.tr_sign = tr_sg;
  r.prob = prob;
  r.rand = rnd;
  if (rnd < prob) {
    for (int q = 0; q < 2; ++q) {
      const int f = q == 0 ? fa : fb;
      if (q == 1 && fb == fa) break;
      const int k = knew[f];
      const double* src = minv_new + (size_t)f * c.kcap * c.kcap;
      double* Mf = M_ptr(c, f);
      for (int e = c.lane; e < k * k; e += 32) {
        const size_t idx = (size_t)(e / k) * c.kcap + (e % k);
        Mf[idx] = src[idx];
      }
      for (int ca = 0; ca < 2; ++ca) {
        const double* st = srt_new + (size_t)(2 * f + ca) * c.kcap;
        for (int i = c.lane; i < k; i += 32) {
          srt_ptr(c, f, ca)[i] = st[i];
          sslot_ptr(c, f, ca)[i] = (short)i;
          stau_ptr(c, f, ca)[i] = st[i];
        }
      }
    }
    __syncwarp();
    tree_flip_all(c);
    if (c.g->o_chk) chk_invalidate(c);
    if (c.lane == 0) {
      h.k[fa] = knew[fa];
      h.k[fb] = knew[fb];
      h.det_log = h.det_log + det_lg;
      h.det_sign = h.det_sign * det_sg;
      h.trace_log = tr_lg;
      h.trace_sign = tr_sg;
      h.npairs = np_new;
    }
    __syncwarp();
    const double sgn = config_sign(c);
    if (c.lane == 0) h.cfgsign = -sgn;
    __syncwarp();
    return 4;
  }
  // restore the present arrays
  const double* tau_old = glob_optau(c);
  const int* opc_old = glob_opcode(c);
  for (int i = c.lane; i < K_old; i += 32) {
    c.optau[i] = tau_old[i];
    c.opcode[i] = opc_old[i];
  }
  if (c.lane == 0) h.K = K_old;
  __syncwarp();
  bstart_build(c);
  return 3;
}

// The same for off-diagonal hybridisation: the full matrix of the proposed
// arrays in block order inverted by Gauss-Jordan, DetRat = DetNew / Det
// (full_rebuild of StepAdd4 / StepRem4 with get_FullHybr_offdiag,
// CTQMC.F90:3822-3827, 4352-4357), the trace from the rebuilt tree, the
// Metropolis draw, installation or the old arrays back.
__device__ NOINL bool od_full_inverse(Ctx& c, int K, double& dlog, double& dsign);
__device__ NOINL void od_trace(Ctx& c, int s0, double& lg, double& sg);
__device__ NOINL int count_pairs_od(Ctx& c);
__device__ NOINL void od_restore(Ctx& c, int K);
__device__ NOINL void od_accept(Ctx& c, double det_lg, double det_sg, double tr_lg, double tr_sg, int new_outer,
                                int np_new);
__device__ NOINL int rebuild4_decide_od(Ctx& c, double factor, int K_old, int np_new) {
  Hdr& h = *c.h;
  cthyb_record& r = *c.rec;
  const int K = h.K, k = K / 2, ld = c.kcap;
  double dlog = 0.0, dsign = 1.0;
  const bool singular = !od_full_inverse(c, K, dlog, dsign);
  double* Mn = glob_minv(c);  // the new inverse (the trace below reuses the dense work space)
  const double* I = c.dense + (size_t)ld * ld;
  for (int e = c.lane; e < k * k && !singular; e += 32) {
    const size_t idx = (size_t)(e / k) * ld + (e % k);
    Mn[idx] = I[idx];
  }
  __syncwarp();
  const double det_lg = singular ? -DHUGE : dlog - h.det_log;
  const double det_sg = singular ? 0.0 : dsign * h.det_sign;
  double tr_lg = -DHUGE, tr_sg = 0.0, prob = 0.0;
  if (!singular) {
    od_trace(c, h.outer_sst, tr_lg, tr_sg);
    prob = fabs(__dmul_rn(factor, exp(__dsub_rn(tr_lg, h.trace_log) + det_lg)));
  }
  const double rnd = grnd(c);
  r.det_log = det_lg;
  r.det_sign = det_sg;
  r.tr_log = tr_lg;
  r.tr_sign = tr_sg;
  r.prob = prob;
  r.rand = rnd;
  if (rnd < prob) {
    double* Mw = M_ptr(c, 0);
    for (int e = c.lane; e < k * k; e += 32) {
      const size_t idx = (size_t)(e / k) * ld + (e % k);
      Mw[idx] = Mn[idx];
    }
    __syncwarp();
    od_accept(c, det_lg, det_sg, tr_lg, tr_sg, h.outer_sst, np_new);
    return 4;
  }
  od_restore(c, K_old);
  return 3;
}

// StepAdd4, CTQMC.F90:3615-3890.
__device__ NOINL void ph_add4(Ctx& c, Prop& p) {
  Hdr& h = *c.h;
  const DModel& m = *c.m;
  cthyb_record& r = *c.rec;
  if (c.lane == 0) h.try_add4++;
  __syncwarp();
  const int K = h.K;
  const double wmin = h.tauwin_min, wmax = h.tauwin_max, tdm = h.taudiff_max;
  // pair_OperAdd with N = 4, force_diagonal (Trace.F90:3657-3702); each
  // pair in time order (process_OperAdd)
  double nt[4];
  int nc[4];
  double tdf = 1.0;
  for (int pr = 0; pr < 2; ++pr) {
    const double w = __dsub_rn(wmax, wmin);
    const double tref = __dadd_rn(wmin, __dmul_rn(w, grnd(c)));
    tdf = __dmul_rn(tdf, w);
    const int orb = randint(c, 1, m.nd);
    const int spin = randint(c, 1, 2);
    const double tmin = fmax(__dsub_rn(tref, tdm), wmin);
    const double w2 = __dsub_rn(fmin(__dadd_rn(tref, tdm), wmax), tmin);
    const double tcr = __dadd_rn(tmin, __dmul_rn(w2, grnd(c)));
    tdf = __dmul_rn(tdf, w2);
    const int f = 2 * (orb - 1) + (spin - 1);
    int fcr = f;  // the creator's flavour: drawn as well with off-diagonal hybridisation
    if (c.g->offdiag) {
      const int orb_c = randint(c, 1, m.nd);
      const int spin_c = randint(c, 1, 2);
      fcr = 2 * (orb_c - 1) + (spin_c - 1);
    }
    const bool afirst = tref < tcr;
    nt[2 * pr] = afirst ? tref : tcr;
    nc[2 * pr] = afirst ? 2 * f + 1 : 2 * fcr;
    nt[2 * pr + 1] = afirst ? tcr : tref;
    nc[2 * pr + 1] = afirst ? 2 * fcr : 2 * f + 1;
  }
  const int fa = nc[0] >> 1, fb = nc[2] >> 1;
  r.orb = fa + 1;
  r.spin = fb + 1;
  r.tau_c = nt[0];
  r.tau_a = nt[1];
  const int dk = fa == fb ? 2 : 1;
  if (K + 4 > c.g->opcap ||
      (c.g->offdiag ? K / 2 + 2 > c.kcap : (h.k[fa] + dk > c.kcap || h.k[fb] + dk > c.kcap))) {
    set_status(c, ST_CAPACITY);
    return;
  }
  // equal times among the new operators or with present ones
  bool equal = nt[0] == nt[1] || nt[0] == nt[2] || nt[0] == nt[3] || nt[1] == nt[2] || nt[1] == nt[3] ||
               nt[2] == nt[3];
  for (int i = c.lane; i < K; i += 32) {
    const double t = c.optau[i];
    equal = equal || t == nt[0] || t == nt[1] || t == nt[2] || t == nt[3];
  }
  equal = __any_sync(FULL, equal);
  if (h.npairs == -1) {  // ensure_valid_NPairs
    const int np = c.g->offdiag ? count_pairs_od(c) : count_npairs(c);
    if (c.lane == 0) h.npairs = np;
    __syncwarp();
  }
  if (equal) {
    r.outcome = 0;
    __syncwarp();
    return;
  }
  // superstates around the changed segment in the present configuration
  const double t_first = fmin(nt[0], nt[2]), t_last = fmax(nt[1], nt[3]);
  const int bs = old_prefix(c, h.outer_sst, t_first);
  const int es = old_prefix(c, h.outer_sst, t_last);
  // proposed arrays: merge the four operators in
  double* tau_old = glob_optau(c);
  int* opc_old = glob_opcode(c);
  for (int i = c.lane; i < K; i += 32) {
    tau_old[i] = c.optau[i];
    opc_old[i] = c.opcode[i];
  }
  __syncwarp();
  int q[4];
  for (int j = 0; j < 4; ++j) {
    int rank = 0;
    for (int l = 0; l < 4; ++l) rank += nt[l] < nt[j];
    q[j] = wlb(tau_old, K, nt[j], c.lane) + rank;
  }
  for (int i = c.lane; i < K; i += 32) {
    const double t = tau_old[i];
    const int d = (nt[0] < t) + (nt[1] < t) + (nt[2] < t) + (nt[3] < t);
    c.optau[i + d] = t;
    c.opcode[i + d] = opc_old[i];
  }
  if (c.lane < 4) {
    c.optau[q[c.lane]] = nt[c.lane];
    c.opcode[q[c.lane]] = nc[c.lane];
  }
  if (c.lane == 0) h.K = K + 4;
  __syncwarp();
  const int Kn = K + 4;
  const int none[4] = {-1, -1, -1, -1};
  const int s12[4] = {q[2], q[3], -1, -1}, s34[4] = {q[0], q[1], -1, -1};
  const int np_12 = count_pairs_skip(c, c.optau, c.opcode, Kn, s12);
  const int np_34 = count_pairs_skip(c, c.optau, c.opcode, Kn, s34);
  const int np_all = count_pairs_skip(c, c.optau, c.opcode, Kn, none);
  double rf;
  int branch = 0;
  if (rempair4(c, h, nt[0], nc[0], nt[3], nc[3]) && rempair4(c, h, nt[1], nc[1], nt[2], nc[2])) {
    branch = 1;
    const int sa[4] = {q[0], q[3], -1, -1}, sb[4] = {q[1], q[2], -1, -1};
    const int np_23 = count_pairs_skip(c, c.optau, c.opcode, Kn, sa);
    const int np_14 = count_pairs_skip(c, c.optau, c.opcode, Kn, sb);
    rf = __dmul_rn(__ddiv_rn(1.0, (double)np_all),
                   __dadd_rn(__dadd_rn(__dadd_rn(__ddiv_rn(1.0, (double)np_12), __ddiv_rn(1.0, (double)np_34)),
                                       __ddiv_rn(1.0, (double)np_14)),
                             __ddiv_rn(1.0, (double)np_23)));
    tdf = __ddiv_rn(tdf, 4.0);
  } else if (rempair4(c, h, nt[0], nc[0], nt[2], nc[2]) && rempair4(c, h, nt[1], nc[1], nt[3], nc[3])) {
    branch = 2;
    const int sa[4] = {q[0], q[2], -1, -1}, sb[4] = {q[1], q[3], -1, -1};
    const int np_23 = count_pairs_skip(c, c.optau, c.opcode, Kn, sa);
    const int np_14 = count_pairs_skip(c, c.optau, c.opcode, Kn, sb);
    rf = __dmul_rn(__ddiv_rn(1.0, (double)np_all),
                   __dadd_rn(__dadd_rn(__dadd_rn(__ddiv_rn(1.0, (double)np_12), __ddiv_rn(1.0, (double)np_34)),
                                       __ddiv_rn(1.0, (double)np_14)),
                             __ddiv_rn(1.0, (double)np_23)));
    tdf = __ddiv_rn(tdf, 4.0);
  } else {
    rf = __dmul_rn(__ddiv_rn(1.0, (double)np_all),
                   __dadd_rn(__ddiv_rn(1.0, (double)np_12), __ddiv_rn(1.0, (double)np_34)));
    tdf = __ddiv_rn(tdf, 2.0);
  }
  r.change_outer = branch;
  r.fpos_c = np_12;
  r.fpos_a = np_34;
  r.npairs = np_all;
  // check_sst_sequence over the merged arrays from the earliest to the
  // latest new operator
  const int first = min(q[0], q[2]), last = max(q[1], q[3]);
  const int w = bs < 0 ? -1 : walk_ops(c, bs, first, last + 1, none);
  if (bs < 0 || w < 0 || w != es) {
    for (int i = c.lane; i < K; i += 32) {
      c.optau[i] = tau_old[i];
      c.opcode[i] = opc_old[i];
    }
    if (c.lane == 0) h.K = K;
    __syncwarp();
    r.outcome = 1;
    __syncwarp();
    return;
  }
  // taudiff_factor * (2 NBands)**2 * rempair_factor, left to right; (2
  // NBands)**4 with off-diagonal hybridisation (both flavours of both pairs
  // drawn, CTQMC.F90:3822-3827)
  const double n2 = 2.0 * m.nd;
  const double fl = c.g->offdiag ? __dmul_rn(__dmul_rn(__dmul_rn(n2, n2), n2), n2) : __dmul_rn(n2, n2);
  const double factor = __dmul_rn(__dmul_rn(tdf, fl), rf);
  r.outcome = c.g->offdiag ? rebuild4_decide_od(c, factor, K, np_all) : rebuild4_decide(c, fa, fb, factor, K, np_all);
  if (r.outcome == 4 && c.lane == 0) h.acc_add4++;
  r.outer_sst = h.outer_sst;
  r.k_total = h.K;
  __syncwarp();
}

// StepRem4, CTQMC.F90:4153-4431.
__device__ NOINL void ph_rem4(Ctx& c, Prop& p) {
  Hdr& h = *c.h;
  const DModel& m = *c.m;
  cthyb_record& r = *c.rec;
  if (c.lane == 0) h.try_rem4++;
  __syncwarp();
  const int K = h.K;
  if (h.npairs == -1) {
    const int np = c.g->offdiag ? count_pairs_od(c) : count_npairs(c);
    if (c.lane == 0) h.npairs = np;
    __syncwarp();
  }
  const int np_old = h.npairs;
  if (np_old <= 0) {
    r.outcome = 2;
    __syncwarp();
    return;
  }
  const int none[4] = {-1, -1, -1, -1};
  int a1, a2;
  if (!select_pair_skip(c, c.optau, c.opcode, K, none, randint(c, 1, np_old), a1, a2)) {
    set_status(c, ST_INTERNAL);
    return;
  }
  const double ta1 = c.optau[a1], ta2 = c.optau[a2];
  const int ca1 = c.opcode[a1], ca2 = c.opcode[a2];
  const double f1 = remfac4(h, np_old, (ca1 & 1) ? ta1 : ta2);
  const int sA[4] = {a1, a2, -1, -1};
  const int np_34 = count_pairs_skip(c, c.optau, c.opcode, K, sA);
  if (np_34 <= 0) {
    r.outcome = 2;
    __syncwarp();
    return;
  }
  int b1, b2;
  if (!select_pair_skip(c, c.optau, c.opcode, K, sA, randint(c, 1, np_34), b1, b2)) {
    set_status(c, ST_INTERNAL);
    return;
  }
  const double tb1 = c.optau[b1], tb2 = c.optau[b2];
  const int cb1 = c.opcode[b1], cb2 = c.opcode[b2];
  const double f2 = remfac4(h, np_34, (cb1 & 1) ? tb1 : tb2);
  double tdf = __ddiv_rn(__ddiv_rn(__dmul_rn((double)np_old, (double)np_34), f1), f2);
  const int sB[4] = {b1, b2, -1, -1};
  const int np_12 = count_pairs_skip(c, c.optau, c.opcode, K, sB);
  double rf;
  int branch = 0;
  if (rempair4(c, h, ta1, ca1, tb2, cb2) && rempair4(c, h, ta2, ca2, tb1, cb1)) {
    branch = 1;
    const int sa[4] = {a1, b2, -1, -1}, sb[4] = {a2, b1, -1, -1};
    const int np_23 = count_pairs_skip(c, c.optau, c.opcode, K, sa);
    const int np_14 = count_pairs_skip(c, c.optau, c.opcode, K, sb);
    rf = __dmul_rn(__ddiv_rn(1.0, (double)np_old),
                   __dadd_rn(__dadd_rn(__dadd_rn(__ddiv_rn(1.0, (double)np_12), __ddiv_rn(1.0, (double)np_34)),
                                       __ddiv_rn(1.0, (double)np_14)),
                             __ddiv_rn(1.0, (double)np_23)));
    tdf = __ddiv_rn(tdf, 4.0);
  } else if (rempair4(c, h, ta1, ca1, tb1, cb1) && rempair4(c, h, ta2, ca2, tb2, cb2)) {
    branch = 2;
    const int sa[4] = {a1, b1, -1, -1}, sb[4] = {a2, b2, -1, -1};
    const int np_23 = count_pairs_skip(c, c.optau, c.opcode, K, sa);
    const int np_14 = count_pairs_skip(c, c.optau, c.opcode, K, sb);
    rf = __dmul_rn(__ddiv_rn(1.0, (double)np_old),
                   __dadd_rn(__dadd_rn(__dadd_rn(__ddiv_rn(1.0, (double)np_12), __ddiv_rn(1.0, (double)np_34)),
                                       __ddiv_rn(1.0, (double)np_14)),
                             __ddiv_rn(1.0, (double)np_23)));
    tdf = __ddiv_rn(tdf, 4.0);
  } else {
    rf = __dmul_rn(__ddiv_rn(1.0, (double)np_old),
                   __dadd_rn(__ddiv_rn(1.0, (double)np_12), __ddiv_rn(1.0, (double)np_34)));
    tdf = __ddiv_rn(tdf, 2.0);
  }
  const int fa = ca1 >> 1, fb = cb1 >> 1;
  r.orb = fa + 1;
  r.spin = fb + 1;
  r.tau_c = ta1;
  r.tau_a = ta2;
  r.change_outer = branch;
  r.fpos_c = np_12;
  r.fpos_a = np_34;
  const int gone[4] = {a1, a2, b1, b2};
  const int np_new = count_pairs_skip(c, c.optau, c.opcode, K, gone);
  r.npairs = np_new;
  // check_sst_sequence over the operators left between the earliest and the
  // latest removed one
  const int first = min(a1, b1), last = max(a2, b2);
  const int bs = old_prefix(c, h.outer_sst, c.optau[first]);
  int es = old_prefix(c, h.outer_sst, c.optau[last]);
  if (es >= 0) {
    const int code = c.opcode[last];
    es = m.connect[((size_t)es * m.nf + (code >> 1)) * 2 + (code & 1)];
  }
  const int w = bs < 0 ? -1 : walk_ops(c, bs, first + 1, last, gone);
  if (bs < 0 || es < 0 || w < 0 || w != es) {
    r.outcome = 1;
    __syncwarp();
    return;
  }
  // proposed arrays without the four operators
  double* tau_old = glob_optau(c);
  int* opc_old = glob_opcode(c);
  for (int i = c.lane; i < K; i += 32) {
    tau_old[i] = c.optau[i];
    opc_old[i] = c.opcode[i];
  }
  __syncwarp();
  for (int i = c.lane; i < K; i += 32) {
    if (i == a1 || i == a2 || i == b1 || i == b2) continue;
    const int d = (a1 < i) + (a2 < i) + (b1 < i) + (b2 < i);
    c.optau[i - d] = tau_old[i];
    c.opcode[i - d] = opc_old[i];
  }
  if (c.lane == 0) h.K = K - 4;
  __syncwarp();
  const double n2 = 2.0 * m.nd;  // (2 NBands)**4 with off-diagonal hybridisation (CTQMC.F90:4352-4357)
  const double fl = c.g->offdiag ? __dmul_rn(__dmul_rn(__dmul_rn(n2, n2), n2), n2) : __dmul_rn(n2, n2);
  const double factor = __ddiv_rn(__ddiv_rn(__ddiv_rn(1.0, fl), tdf), rf);
  r.outcome = c.g->offdiag ? rebuild4_decide_od(c, factor, K, np_new) : rebuild4_decide(c, fa, fb, factor, K, np_new);
  if (r.outcome == 4 && c.lane == 0) h.acc_rem4++;
  r.outer_sst = h.outer_sst;
  r.k_total = h.K;
  __syncwarp();
}

// ---------------------------------------------------------------------------
// Off-diagonal hybridisation (offdiag = 1): StepAdd / StepRem with
// unconstrained flavours (pair_OperAdd force_diagonal = .false.,
// Trace.F90:3657-3702), F for every flavour pair (get_HybrF_full), one
// inverse matrix over all flavours in the reference's block order
// (flavour-major, time within a flavour; rows creators, columns
// annihilators; get_LogDetRatPairAdd_full / get_LogDetRatPairRem_full with
// add_ftau_offset, Trace.F90:2835-3040), removable pairs of any flavours
// (Trace.F90:1818-1992), (2 Nd)^2 proposal factors (CTQMC.F90:3517-3523,
// 4050-4056) and the configuration sign of recalc_sign (Trace.F90:3479-3545).
// These proposals run in the rare-move phase: the proposed operator arrays
// are written in place (old ones saved in the o_glob space), the tree is
// rebuilt into the inactive slots and the full trace taken from it; the
// determinant ratio is the fast S - R.M.Q over the full matrix, whose
// accepted update inserts or removes one row and column in block order.

// get_HybrF_full(tau; f1, f2)
__device__ __forceinline__ double hybrf_full(const Ctx& c, double tau, int f1, int f2) {
  const DGroup& g = *c.g;
  const long long neg = __double_as_longlong(tau) & (long long)0x8000000000000000ll;
  if (neg) tau = tau + g.beta;
  const double n = tau * g.hscale;
  const int in = (int)n;
  const double fr = n - (double)in;
  const int i = min(max(in, 0), g.nftau - 2);
  const double* F = g.hybr_full + ((size_t)f1 * c.m->nf + f2) * g.nftau;
  const double f0 = __ldg(F + i), f1v = __ldg(F + i + 1);
  const double v = fma(fr, f1v - f0, f0);
  return __longlong_as_double(__double_as_longlong(v) ^ neg);
}

__device__ __forceinline__ int conn_code(const DModel& m, int s, int code) {
  return s < 0 ? -1 : m.connect[((size_t)s * m.nf + (code >> 1)) * 2 + (code & 1)];
}

// 1-based block position a new operator (code 2f + ca, time t) would take
// among the present operators of its kind (creators ca 0, annihilators 1).
__device__ NOINL int od_pos_new(Ctx& c, int code, double t) {
  const int K = c.h->K, ca = code & 1, f = code >> 1;
  int n = 0;
  for (int j = c.lane; j < K; j += 32) {
    const int cd = c.opcode[j];
    if ((cd & 1) != ca) continue;
    const int fj = cd >> 1;
    n += fj < f || (fj == f && c.optau[j] < t);
  }
  return wsumi(n) + 1;
}

// Block position (0-based) of every present operator into pos[0..K).
__device__ NOINL void od_positions(Ctx& c, int* pos) {
  const int K = c.h->K, ncode = 2 * c.m->nf;
  const unsigned lt = (1u << c.lane) - 1u;
  int cnt[2 * NFMAX];
  for (int q = 0; q < ncode; ++q) cnt[q] = 0;
  for (int base = 0; base < K; base += 32) {  // operators of each code
    const int i = base + c.lane;
    const int mc = i < K ? c.opcode[i] : -1;
    for (int q = 0; q < ncode; ++q) cnt[q] += __popc(__ballot_sync(FULL, mc == q));
  }
  int off[2 * NFMAX];  // block offset of each code: earlier flavours of the same kind
  for (int q = 0; q < ncode; ++q) {
    off[q] = 0;
    for (int r = q & 1; r < q; r += 2) off[q] += cnt[r];
  }
  int run[2 * NFMAX];
  for (int q = 0; q < ncode; ++q) run[q] = 0;
  for (int base = 0; base < K; base += 32) {
    const int i = base + c.lane;
    const int mc = i < K ? c.opcode[i] : -1;
    for (int q = 0; q < ncode; ++q) {
      const unsigned bal = __ballot_sync(FULL, mc == q);
      if (mc == q) pos[i] = off[q] + run[q] + __popc(bal & lt);
      run[q] += __popc(bal);
    }
  }
  __syncwarp();
}

// Removable pairs of any flavours in the present arrays
// (ensure_valid_NPairs_offdiag, Trace.F90:1818-1856).
__device__ NOINL int count_pairs_od(Ctx& c) {
  const Hdr& h = *c.h;
  const int K = h.K;
  int tot = 0;
  for (int i = c.lane; i < K; i += 32) {
    const double x = c.optau[i];
    if (x < h.tauwin_min || x > h.tauwin_max) continue;
    const int cx = c.opcode[i] & 1;
    const double hi = fmin(h.tauwin_max, __dadd_rn(x, h.taudiff_max));
    for (int j = i + 1; j < K; ++j) {
      if (c.optau[j] > hi) break;
      tot += (c.opcode[j] & 1) != cx;
    }
  }
  return wsumi(tot);
}

// The target-th removable pair (1-based) in the scan order of gen_OperRemove
// with off-diagonal hybridisation (Trace.F90:4880-4910): ix < iy.
__device__ NOINL bool select_pair_od(Ctx& c, int target, int& ix, int& iy) {
  const Hdr& h = *c.h;
  const int K = h.K;
  const double wmin = h.tauwin_min, wmax = h.tauwin_max, tdm = h.taudiff_max;
  const int start = wlb(c.optau, K, wmin, c.lane);
  for (int base = start; base < K; base += 32) {
    const int i = base + c.lane;
    int cnt = 0;
    if (i < K) {
      const int cx = c.opcode[i] & 1;
      const double hi = fmin(wmax, __dadd_rn(c.optau[i], tdm));
      for (int j = i + 1; j < K; ++j) {
        if (c.optau[j] > hi) break;
        cnt += (c.opcode[j] & 1) != cx;
      }
    }
    int cum = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(FULL, cum, o);
      if (c.lane >= o) cum += y;
    }
    const int total = __shfl_sync(FULL, cum, 31);
    if (target <= total) {
      const unsigned bal = __ballot_sync(FULL, cum >= target);
      const int L0 = __ffs(bal) - 1;
      const int before = __shfl_sync(FULL, cum - cnt, L0);
      int jy = -1;
      if (c.lane == L0) {
        int want = target - before;
        const int cx = c.opcode[i] & 1;
        const double hi = fmin(wmax, __dadd_rn(c.optau[i], tdm));
        for (int j = i + 1; j < K; ++j) {
          if (c.optau[j] > hi) break;
          if ((c.opcode[j] & 1) != cx && --want <= 0) {
            jy = j;
            break;
          }
        }
      }
      ix = base + L0;
      iy = __shfl_sync(FULL, jy, L0);
      return iy > ix;
    }
    target -= total;
  }
  return false;
}

// Configuration sign with off-diagonal hybridisation: -(trace sign x
// determinant sign x recalc_sign).  recalc_sign's double loop sorts the keys
// (3 - CA) * 100000 + Orbital * 10000 + Spin * 1000 + tau descending, so its
// exchange count has the parity of the number of ascending key pairs; to it
// the loop adds sum_{i < n/2} i.
__device__ __forceinline__ double od_key(const Ctx& c, int j) {
  const int cd = c.opcode[j], f = cd >> 1;
  const double a = (double)(2 - (cd & 1)) * 100000.0 + (double)((f >> 1) + 1) * 10000.0 + (double)((f & 1) + 1) * 1000.0;
  return __dadd_rn(a, c.optau[j]);
}
__device__ NOINL double od_cfgsign(Ctx& c) {
  const Hdr& h = *c.h;
  const int K = h.K;
  int asc = 0;
  for (int i = c.lane; i < K; i += 32) {
    const double ki = od_key(c, i);
    for (int j = i + 1; j < K; ++j) asc += ki < od_key(c, j);
  }
  asc = wsumi(asc);
  const long long half = K / 2;
  const long long perm = (long long)asc + (half >= 2 ? (half - 1) * half / 2 : 0);
  const double rs = (perm & 1) ? -1.0 : 1.0;
  return -(h.trace_sign * h.det_sign * rs);
}

// The present operator arrays back from their copy in the o_glob space.
__device__ NOINL void od_restore(Ctx& c, int K) {
  const double* t = glob_optau(c);
  const int* o = glob_opcode(c);
  for (int i = c.lane; i < K; i += 32) {
    c.optau[i] = t[i];
    c.opcode[i] = o[i];
  }
  if (c.lane == 0) c.h->K = K;
  __syncwarp();
  bstart_build(c);
}

// Trace of the proposed arrays with outer superstate s0 from a full rebuild
// of the tree into the inactive slots.
__device__ NOINL void od_trace(Ctx& c, int s0, double& lg, double& sg) {
  bstart_build(c);
  tree_build_inactive(c, true, false);
  rebuilt_trace(c, s0, lg, sg);
}

// Installation of an accepted off-diagonal move: tree, weights, sign.
__device__ NOINL void od_accept(Ctx& c, double det_lg, double det_sg, double tr_lg, double tr_sg, int new_outer,
                                int np_new) {
  Hdr& h = *c.h;
  tree_flip_all(c);
  if (c.g->o_chk) chk_invalidate(c);
  if (c.lane == 0) {
    h.det_log = h.det_log + det_lg;
    h.det_sign = h.det_sign * det_sg;
    h.trace_log = tr_lg;
    h.trace_sign = tr_sg;
    h.outer_sst = new_outer;
    h.npairs = np_new;
    h.acc_since_refresh++;
  }
  __syncwarp();
  const double cs = od_cfgsign(c);
  if (c.lane == 0) h.cfgsign = cs;
  __syncwarp();
}

// Off-diagonal pair moves evaluate the proposed configuration like the
// diagonal ones: the two changed leaves of the time-bin tree and their
// ancestors are rebuilt into the inactive slots (quantum numbers from the
// superstate maps, the trace from the state maps or the dense-block
// checkpoints), and the operator arrays change only on acceptance.

// Quantum-number check of the proposal md (check_sst_sequence,
// Trace.F90:1243-1304) on the proposed superstate tree; snew: the outer
// superstate of the proposed configuration (a new one with change_outer).
__device__ NOINL bool od_tree_qn(Ctx& c, Mod& md, bool co, int& snew) {
  tree_propose(c, md, true, false, true);
  const int root_new = 1 - c.act[1];
  const int s0 = c.h->outer_sst;
  snew = s0;
  if (!co) return node_ss(c, 1, root_new)[s0] == s0;
  const int inside = old_prefix(c, s0, md.t2);
  snew = inside >= 0 ? new_suffix(c, md, inside, md.t2) : -1;
  return snew >= 0 && node_ss(c, 1, root_new)[snew] == snew;
}

// Removable pairs (update_NPairs with off-diagonal hybridisation) that the
// two operators of an insertion add: present operators of the other kind
// (creator/annihilator, any flavour) whose earlier member lies in the window
// and whose later member lies within TaudiffMax of it and inside the
// window, and the inserted pair itself.
__device__ NOINL int od_new_pairs(Ctx& c, const Mod& md) {
  const Hdr& h = *c.h;
  const double wmin = h.tauwin_min, wmax = h.tauwin_max, tdm = h.taudiff_max;
  int n = 0;
  for (int i = c.lane; i < h.K; i += 32) {
    const double t = c.optau[i];
    const int ca = c.opcode[i] & 1;
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const double tn = q ? md.t2 : md.t1;
      if (((q ? md.c2 : md.c1) & 1) == ca) continue;
      const double e = fmin(t, tn), l = fmax(t, tn);
      n += e >= wmin && e <= wmax && l <= fmin(wmax, __dadd_rn(e, tdm));
    }
  }
  n = wsumi(n);
  return n + (md.t1 >= wmin && md.t1 <= wmax && md.t2 <= fmin(wmax, __dadd_rn(md.t1, tdm)));
}

// Installation of an accepted off-diagonal pair move whose operator arrays,
// inverse matrix and bin starts are already updated: tree flip of the
// changed path, checkpoints, weights, pairs, sign.
__device__ NOINL void od_accept_pair(Ctx& c, const Mod& md, double det_lg, double det_sg, double tr_lg,
                                     double tr_sg, int new_outer, int np_new) {
  Hdr& h = *c.h;
  tree_accept(c, md);
  chk_keep(c, md, new_outer);
  if (c.lane == 0) {
    h.det_log = h.det_log + det_lg;
    h.det_sign = h.det_sign * det_sg;
    h.trace_log = tr_lg;
    h.trace_sign = tr_sg;
    h.outer_sst = new_outer;
    h.npairs = np_new;
    h.acc_since_refresh++;
  }
  __syncwarp();
  const double cs = od_cfgsign(c);
  if (c.lane == 0) h.cfgsign = cs;
  __syncwarp();
}

// StepAdd, CTQMC.F90:3353-3613, off-diagonal branch.
__device__ NOINL void ph_add_od(Ctx& c, Prop& p) {
  Hdr& h = *c.h;
  const DModel& m = *c.m;
  cthyb_record& r = *c.rec;
  const int K = h.K;
  const double wmin = h.tauwin_min, wmax = h.tauwin_max, tdm = h.taudiff_max;
  // pair_OperAdd(force_diagonal = .false.): the annihilator at tau_ref with
  // its own orbital and spin, then the creator within TaudiffMax with its own
  const double w = __dsub_rn(wmax, wmin);
  const double tau_a = __dadd_rn(wmin, __dmul_rn(w, grnd(c)));
  double tdf = __dmul_rn(1.0, w);
  const int orb_a = randint(c, 1, m.nd);
  const int spin_a = randint(c, 1, 2);
  const double tmin = fmax(__dsub_rn(tau_a, tdm), wmin);
  const double w2 = __dsub_rn(fmin(__dadd_rn(tau_a, tdm), wmax), tmin);
  const double tau_c = __dadd_rn(tmin, __dmul_rn(w2, grnd(c)));
  tdf = __dmul_rn(tdf, w2);
  const int orb_c = randint(c, 1, m.nd);
  const int spin_c = randint(c, 1, 2);
  const int fa = 2 * (orb_a - 1) + (spin_a - 1), fc = 2 * (orb_c - 1) + (spin_c - 1);
  const int code_a = 2 * fa + 1, code_c = 2 * fc;
  r.orb = fc + 1;
  r.spin = fa + 1;
  r.tau_c = tau_c;
  r.tau_a = tau_a;
  const int k = K / 2;
  if (K + 2 > c.g->opcap || k + 1 > c.kcap) {
    set_status(c, ST_CAPACITY);
    return;
  }
  const bool afirst = tau_a < tau_c;
  Mod& md = p.md;
  md.type = 1;
  md.t1 = afirst ? tau_a : tau_c;
  md.t2 = afirst ? tau_c : tau_a;
  md.c1 = afirst ? code_a : code_c;
  md.c2 = afirst ? code_c : code_a;
  md.ix = md.iy = -1;
  md.b1 = bin_of(c, md.t1);
  md.b2 = bin_of(c, md.t2);
  const int p1 = op_lower_bound(c, md.b1, md.t1), p2 = op_lower_bound(c, md.b2, md.t2);
  md.p1 = p1;
  md.p2 = p2;
  if (teq(tau_a, tau_c) || (p1 < K && teq(c.optau[p1], md.t1)) || (p2 < K && teq(c.optau[p2], md.t2))) {
    if (c.lane == 0) h.qn_add++;
    r.outcome = 0;
    __syncwarp();
    return;
  }
  const int pos_c = od_pos_new(c, code_c, tau_c), pos_a = od_pos_new(c, code_a, tau_a);
  r.fpos_c = pos_c;
  r.fpos_a = pos_a;
  int snew;
  if (!od_tree_qn(c, md, p.co, snew)) {
    if (c.lane == 0) h.qn_add++;
    r.outcome = 1;
    __syncwarp();
    return;
  }
  if (c.mono) tree_propose(c, md, false, true, false);
  double tr_mx, tr_sum;
  proposed_trace(c, md, snew, tr_mx, tr_sum, solo_team(c));
  // determinant ratio S - R.M.Q over the full matrix; Q over the present
  // annihilators with the flavour pair (creator, annihilator) as the
  // reference passes it (Trace.F90:2892), R over the present creators
  // (the block positions reuse the gathered-leaf buffer, no longer needed)
  double* Q = c.scr;
  double* R = c.scr + c.kcap;
  double* v = c.scr + 2 * c.kcap;
  double* wv = c.scr + 3 * c.kcap;
  int* pos = c.bcode[1];
  od_positions(c, pos);
  for (int i = c.lane; i < K; i += 32) {
    const int cd = c.opcode[i], fi = cd >> 1;
    const double t = c.optau[i];
    if (cd & 1) Q[pos[i]] = hybrf_full(c, __dsub_rn(t, tau_c), fc, fi);
    else R[pos[i]] = hybrf_full(c, __dsub_rn(tau_a, t), fa, fi);
  }
  const double S = hybrf_full(c, __dsub_rn(tau_a, tau_c), fa, fc);
  __syncwarp();
  const double* Mf = M_ptr(c, 0);
  const int ld = c.kcap;
  double part = 0.0;
  for (int i = c.lane; i < k; i += 32) {
    double acc = 0.0;
    for (int j = 0; j < k; ++j) acc = fma(Mf[(size_t)j * ld + i], Q[j], acc);
    v[i] = acc;
    part = fma(R[i], acc, part);
  }
  const double ratio = S - wsum(part);
  const double sig = ((pos_c - pos_a) & 1) ? -1.0 : 1.0;
  const double det_sg = (ratio >= 0.0 ? 1.0 : -1.0) * sig;
  if (c.lane == 0) {
    h.w_mbytes += 8ll * k * k + 32ll * k;
    h.w_mflops += 2ll * k * k + 2ll * k;
  }
  if (h.npairs == -1) {
    const int np = count_pairs_od(c);
    if (c.lane == 0) h.npairs = np;
    __syncwarp();
  }
  const int np_new = h.npairs + od_new_pairs(c, md);
  const double rnd = grnd(c);
  const double n2 = 2.0 * m.nd;
  const double wr = weight_ratio(tr_mx, tr_sum, h.trace_log, fabs(ratio));
  const double prob = fabs(__dmul_rn(__ddiv_rn(__dmul_rn(tdf, __dmul_rn(n2, n2)), (double)np_new), wr));
  const bool accept = rnd < prob;
  double det_lg = 0.0, tr_lg = 0.0, tr_sg = 0.0;
  if (accept || c.log) {
    det_lg = log(fabs(ratio));
    trace_log(tr_mx, tr_sum, tr_lg, tr_sg);
  }
  r.det_log = det_lg;
  r.det_sign = det_sg;
  r.tr_log = tr_lg;
  r.tr_sign = tr_sg;
  r.prob = prob;
  r.rand = rnd;
  r.npairs = np_new;
  if (accept) {
    // get_MatAdd in block order: new row pos_c, new column pos_a
    for (int j = c.lane; j < k; j += 32) {
      double acc = 0.0;
      const double* col = Mf + (size_t)j * ld;
      for (int i = 0; i < k; ++i) acc = fma(R[i], col[i], acc);
      wv[j] = acc;
    }
    __syncwarp();
    double* T = glob_minv(c);
    const int pc = pos_c - 1, pa = pos_a - 1, kn = k + 1;
    const double inv = 1.0 / ratio;
    for (int e = c.lane; e < kn * kn; e += 32) {
      const int in = e % kn, jn = e / kn;
      double val;
      if (in == pc && jn == pa) {
        val = inv;
      } else if (jn == pa) {
        val = -v[in < pc ? in : in - 1] * inv;
      } else if (in == pc) {
        val = -wv[jn < pa ? jn : jn - 1] * inv;
      } else {
        const int io = in < pc ? in : in - 1, jo = jn < pa ? jn : jn - 1;
        val = Mf[(size_t)jo * ld + io] + v[io] * wv[jo] * inv;
      }
      T[(size_t)jn * ld + in] = val;
    }
    __syncwarp();
    double* Mw = M_ptr(c, 0);
    for (int e = c.lane; e < kn * kn; e += 32) {
      const size_t idx = (size_t)(e / kn) * ld + (e % kn);
      Mw[idx] = T[idx];
    }
    if (c.lane == 0) {
      h.w_mbytes += 24ll * kn * kn + 16ll * k * k;
      h.w_mflops += 4ll * kn * kn;
      h.w_opbytes += 24ll * (K - p1);
    }
    __syncwarp();
    ops_insert2(c, p1, p2, md.t1, md.c1, md.t2, md.c2);
    if (c.lane == 0) h.K = K + 2;
    __syncwarp();
    bstart_shift(c, md.b1, md.b2, +1);
    od_accept_pair(c, md, det_lg, det_sg, tr_lg, tr_sg, snew, np_new);
    count_accpair(c, md.c1 >> 1, __dsub_rn(md.t2, md.t1));
    if (c.lane == 0) h.acc_add++;
    r.outcome = 4;
  } else {
    r.outcome = 3;
  }
  r.outer_sst = h.outer_sst;
  r.k_total = h.K;
  __syncwarp();
}

// StepRem, CTQMC.F90:3892-4151, off-diagonal branch.
__device__ NOINL void ph_rem_od(Ctx& c, Prop& p) {
  Hdr& h = *c.h;
  const DModel& m = *c.m;
  cthyb_record& r = *c.rec;
  const int K = h.K;
  if (h.npairs == -1) {
    const int np = count_pairs_od(c);
    if (c.lane == 0) h.npairs = np;
    __syncwarp();
  }
  const int np = h.npairs;
  if (np <= 0) {
    if (c.lane == 0) h.qn_rem++;
    r.outcome = 2;
    __syncwarp();
    return;
  }
  int ix, iy;
  if (!select_pair_od(c, randint(c, 1, np), ix, iy)) {
    set_status(c, ST_INTERNAL);
    return;
  }
  const double tx = c.optau[ix], ty = c.optau[iy];
  const int cx = c.opcode[ix], cy = c.opcode[iy];
  const bool xc = (cx & 1) == 0;  // x is the creator
  const double tau_c = xc ? tx : ty, tau_a = xc ? ty : tx;
  const int code_c = xc ? cx : cy;
  const int fc = code_c >> 1, fa = (xc ? cy : cx) >> 1;
  int* pos = c.bcode[1];
  od_positions(c, pos);
  const int pos_c = pos[xc ? ix : iy] + 1, pos_a = pos[xc ? iy : ix] + 1;
  __syncwarp();
  const double hprf = __ddiv_rn((double)np, __dmul_rn(__dsub_rn(h.tauwin_max, h.tauwin_min),
                                                      __dsub_rn(fmin(__dadd_rn(tau_a, h.taudiff_max), h.tauwin_max),
                                                                fmax(__dsub_rn(tau_a, h.taudiff_max), h.tauwin_min))));
  r.orb = fc + 1;
  r.spin = fa + 1;
  r.tau_c = tau_c;
  r.tau_a = tau_a;
  r.fpos_c = pos_c;
  r.fpos_a = pos_a;
  r.npairs = np;
  Mod& md = p.md;
  md.type = 2;
  md.ix = ix;
  md.iy = iy;
  md.t1 = tx;
  md.t2 = ty;
  md.c1 = md.c2 = 0;
  md.b1 = bin_of(c, tx);
  md.b2 = bin_of(c, ty);
  int snew;
  if (!od_tree_qn(c, md, p.co, snew)) {
    if (c.lane == 0) h.qn_rem++;
    r.outcome = 1;
    __syncwarp();
    return;
  }
  if (c.mono) tree_propose(c, md, false, true, false);
  double tr_mx, tr_sum;
  proposed_trace(c, md, snew, tr_mx, tr_sum, solo_team(c));
  const int k = K / 2, ld = c.kcap, pc = pos_c - 1, pa = pos_a - 1;
  const double* Mf = M_ptr(c, 0);
  const double dr = Mf[(size_t)pa * ld + pc];
  const double sig = ((pos_c - pos_a) & 1) ? -1.0 : 1.0;
  const double det_sg = (dr >= 0.0 ? 1.0 : -1.0) * sig;
  const double n2 = 2.0 * m.nd;
  const double wr = weight_ratio(tr_mx, tr_sum, h.trace_log, fabs(dr));
  const double prob = fabs(__dmul_rn(__ddiv_rn(hprf, __dmul_rn(n2, n2)), wr));
  const double rnd = grnd(c);
  const bool accept = rnd < prob;
  double det_lg = 0.0, tr_lg = 0.0, tr_sg = 0.0;
  if (accept || c.log) {
    det_lg = log(fabs(dr));
    trace_log(tr_mx, tr_sum, tr_lg, tr_sg);
  }
  r.det_log = det_lg;
  r.det_sign = det_sg;
  r.tr_log = tr_lg;
  r.tr_sign = tr_sg;
  r.prob = prob;
  r.rand = rnd;
  if (accept) {
    if (fabs(dr) < 1e-12) {  // CTQMC.F90:4062
      set_status(c, ST_NUMERIC);
      return;
    }
    // get_MatRem in block order: row pos_c and column pos_a leave
    double* T = glob_minv(c);
    const int kn = k - 1;
    const double inv = 1.0 / dr;
    for (int e = c.lane; e < kn * kn; e += 32) {
      const int in = e % kn, jn = e / kn;
      const int io = in < pc ? in : in + 1, jo = jn < pa ? jn : jn + 1;
      T[(size_t)jn * ld + in] = Mf[(size_t)jo * ld + io] - Mf[(size_t)pa * ld + io] * Mf[(size_t)jo * ld + pc] * inv;
    }
    __syncwarp();
    double* Mw = M_ptr(c, 0);
    for (int e = c.lane; e < kn * kn; e += 32) {
      const size_t idx = (size_t)(e / kn) * ld + (e % kn);
      Mw[idx] = T[idx];
    }
    if (c.lane == 0) {
      h.w_mbytes += 24ll * kn * kn + 16ll * kn;
      h.w_mflops += 2ll * kn * kn;
      h.w_opbytes += 24ll * (K - ix);
    }
    __syncwarp();
    ops_remove2(c, ix, iy);
    if (c.lane == 0) h.K = K - 2;
    __syncwarp();
    bstart_shift(c, md.b1, md.b2, -1);
    const int np_new = count_pairs_od(c);
    od_accept_pair(c, md, det_lg, det_sg, tr_lg, tr_sg, snew, np_new);
    count_accpair(c, fc, __dsub_rn(ty, tx));
    if (c.lane == 0) h.acc_rem++;
    r.outcome = 4;
  } else {
    r.outcome = 3;
  }
  r.outer_sst = h.outer_sst;
  r.k_total = h.K;
  __syncwarp();
}

// Legendre coefficients of one G sample: lsum[l] += M P_l(x), P_l by the
// three-term recurrence in the reference's operation order
// (CTQMC.F90:2368-2389, 2533-2555).
__device__ __forceinline__ void legendre_add(double Mv, double x, int nleg, double* lsum) {
  double plx = 0.0, plm1 = 0.0;
  for (int l = 0; l < nleg; ++l) {
    double p;
    if (l == 0) {
      p = 1.0;
    } else if (l == 1) {
      p = x;
    } else {
      const int ll = l - 1;
      p = __dsub_rn(__dmul_rn(__dmul_rn(__ddiv_rn(2.0 * ll + 1.0, (double)(ll + 1)), x), plx),
                    __dmul_rn(__ddiv_rn((double)ll, (double)(ll + 1)), plm1));
    }
    lsum[l] = __dadd_rn(lsum[l], __dmul_rn(Mv, p));
    plm1 = plx;
    plx = p;
  }
}

// MeasGtauRem_full (CTQMC.F90:2475-2584) and MeasExpOrder with
// NOSOper(b,s)/2 = (creators + annihilators of the flavour) / 2.
__device__ NOINL void measure_od(Ctx& c) {
  const Hdr& h = *c.h;
  const DModel& m = *c.m;
  const DGroup& g = *c.g;
  const int K = h.K, nf = m.nf, nt = g.ntau, k = K / 2, ld = c.kcap;
  for (int f = 0; f < nf; ++f) {
    int n = 0;
    for (int i = c.lane; i < K; i += 32) n += (c.opcode[i] >> 1) == f;
    n = wsumi(n) / 2;
    if (c.lane == 0) c.histo[(size_t)f * g.maxhisto + (n < g.maxhisto - 1 ? n : g.maxhisto - 1)] += 1.0;
  }
  __syncwarp();
  if (k == 0) return;
  // times and flavours by block position
  int* pos = c.bcode[1];
  od_positions(c, pos);
  double* ct = c.scr;
  double* at = c.scr + c.kcap;
  int* cf = (int*)(c.scr + 2 * c.kcap);
  int* af = (int*)(c.scr + 3 * c.kcap);
  for (int i = c.lane; i < K; i += 32) {
    const int cd = c.opcode[i];
    if (cd & 1) {
      at[pos[i]] = c.optau[i];
      af[pos[i]] = cd >> 1;
    } else {
      ct[pos[i]] = c.optau[i];
      cf[pos[i]] = cd >> 1;
    }
  }
  __syncwarp();
  double* G = (double*)((char*)c.gtau - g.o_gtau + g.o_gfull);
  const double* Mf = M_ptr(c, 0);
  for (int e = c.lane; e < k * k; e += 32) {
    const int i = e % k, j = e / k;  // creator row i, annihilator column j
    double Mv = Mf[(size_t)j * ld + i];
    const double ta = at[j], tc = ct[i];
    double dt;
    if (ta - tc > 0.0) {
      dt = ta - tc;
    } else {
      dt = g.beta + ta - tc;
      Mv = -Mv;
    }
    const double q = dt * g.gscale;
    int idt = (int)q;
    const double fr = q - (double)idt;
    if (fr < 1e-9 || fr > 1.0 - 1e-9) idt = (int)__dmul_rn(__ddiv_rn(dt, g.beta), (double)nt);
    idt += 1;
    if (idt > nt) idt = nt;
    Mv = Mv * h.cfgsign;
    atomicAdd(&G[((size_t)af[j] * nf + cf[i]) * nt + idt - 1], Mv);
  }
  __syncwarp();
  // GLeg_full (CTQMC.F90:2533-2555): per (annihilator flavour, creator
  // flavour) block of the inverse matrix, lane partial sums reduced over
  // the warp
  const int nleg = g.nleg;
  if (nleg <= 0) return;
  int offc[NFMAX + 1], offa[NFMAX + 1];
  offc[0] = offa[0] = 0;
  for (int f = 0; f < nf; ++f) {
    int nc = 0, na = 0;
    for (int i = c.lane; i < K; i += 32) {
      nc += c.opcode[i] == 2 * f;
      na += c.opcode[i] == 2 * f + 1;
    }
    offc[f + 1] = offc[f] + wsumi(nc);
    offa[f + 1] = offa[f] + wsumi(na);
  }
  double* GL = (double*)((char*)c.gtau - g.o_gtau + g.o_gleg);  // [fa][fc][l]
  double* lsum = (double*)((char*)c.gtau - g.o_gtau + g.o_glscr) + (size_t)c.lane * nleg;
  for (int fa = 0; fa < nf; ++fa)
    for (int fc = 0; fc < nf; ++fc) {
      const int na = offa[fa + 1] - offa[fa], nc = offc[fc + 1] - offc[fc];
      if (na == 0 || nc == 0) continue;
      for (int l = 0; l < nleg; ++l) lsum[l] = 0.0;
      for (int e = c.lane; e < na * nc; e += 32) {
        const int i = offc[fc] + e % nc, j = offa[fa] + e / nc;
        double Mv = Mf[(size_t)j * ld + i];
        const double ta = at[j], tc = ct[i];
        double dt;
        if (ta - tc > 0.0) {
          dt = ta - tc;
        } else {
          dt = g.beta + ta - tc;
          Mv = -Mv;
        }
        legendre_add(Mv * h.cfgsign, __dsub_rn(__dmul_rn(__ddiv_rn(2.0, g.beta), dt), 1.0), nleg, lsum);
      }
      __syncwarp();
      double* dst = GL + ((size_t)fa * nf + fc) * nleg;
      for (int l = 0; l < nleg; ++l) {
        const double v = wsum(lsum[l]);
        if (c.lane == 0) dst[l] += v;
      }
      __syncwarp();
    }
}

// Inverse of the full hybridisation matrix of the configuration in the
// operator arrays (K operators) in block order (get_FullHybr_offdiag,
// Trace.F90:2690-2770, inverted by Gauss-Jordan): on return
// c.dense + kcap^2 holds element (creator position, annihilator position)
// at [a * kcap + c]; log|det| and sign in dlog/dsign.  False when singular.
__device__ NOINL bool od_full_inverse(Ctx& c, int K, double& dlog, double& dsign) {
  const int k = K / 2, ld = c.kcap;
  int* pos = c.bcode[1];
  od_positions(c, pos);
  double* ct = c.scr;
  double* at = c.scr + ld;
  int* cf = (int*)(c.scr + 2 * ld);
  int* af = (int*)(c.scr + 3 * ld);
  for (int i = c.lane; i < K; i += 32) {
    const int cd = c.opcode[i];
    if (cd & 1) {
      at[pos[i]] = c.optau[i];
      af[pos[i]] = cd >> 1;
    } else {
      ct[pos[i]] = c.optau[i];
      cf[pos[i]] = cd >> 1;
    }
  }
  __syncwarp();
  double* H = c.dense;
  double* I = c.dense + (size_t)ld * ld;
  for (int e = c.lane; e < k * k; e += 32) {
    const int ia = e % k, ic = e / k;
    H[(size_t)ic * ld + ia] = hybrf_full(c, __dsub_rn(at[ia], ct[ic]), af[ia], cf[ic]);
    I[(size_t)ic * ld + ia] = ia == ic ? 1.0 : 0.0;
  }
  __syncwarp();
  dlog = 0.0;
  dsign = 1.0;
  return gj_eliminate(c, k, H, I, dlog, dsign);
}

// StepGlob with off-diagonal hybridisation (CTQMC.F90:4491-4494): the full
// hybridisation matrix of the permuted operators in block order
// (get_FullHybr_offdiag, Trace.F90:2690-2770), its inverse and determinant
// (get_MatLogDetFull), DetRat = DetNew / Det; then the trace, the
// Metropolis draw and the installation, or the old codes back.
__device__ NOINL void global_od_tail(Ctx& c, int K, int new_outer, double factor, const int* opc_old) {
  Hdr& h = *c.h;
  cthyb_record& r = *c.rec;
  const int k = K / 2, ld = c.kcap;
  double dlog, dsign;
  const bool singular = !od_full_inverse(c, K, dlog, dsign);
  const double* I = c.dense + (size_t)ld * ld;
  // the new inverse kept in the o_glob space (the dense trace below reuses
  // the dense work space)
  double* Mn = glob_minv(c);
  for (int e = c.lane; e < k * k && !singular; e += 32) {
    const size_t idx = (size_t)(e / k) * ld + (e % k);
    Mn[idx] = I[idx];
  }
  __syncwarp();
  const double det_lg = singular ? -DHUGE : dlog - h.det_log;
  const double det_sg = singular ? 0.0 : dsign * h.det_sign;
  double tr_lg = -DHUGE, tr_sg = 0.0, prob = 0.0;
  if (!singular) {
    rebuilt_trace(c, new_outer, tr_lg, tr_sg);
    prob = fabs(exp(__dsub_rn(tr_lg, h.trace_log) + det_lg) * factor);
  }
  const double rnd = grnd(c);
  r.det_log = det_lg;
  r.det_sign = det_sg;
  r.tr_log = tr_lg;
  r.tr_sign = tr_sg;
  r.prob = prob;
  r.rand = rnd;
  if (rnd < prob) {
    double* Mw = M_ptr(c, 0);
    for (int e = c.lane; e < k * k; e += 32) {
      const size_t idx = (size_t)(e / k) * ld + (e % k);
      Mw[idx] = Mn[idx];
    }
    __syncwarp();
    tree_flip_all(c);
    if (c.g->o_chk) chk_invalidate(c);
    if (c.lane == 0) {
      h.det_log = dlog;
      h.det_sign = dsign;
      h.trace_log = tr_lg;
      h.trace_sign = tr_sg;
      h.outer_sst = new_outer;
      h.acc_glob++;
    }
    __syncwarp();
    const double cs = od_cfgsign(c);
    if (c.lane == 0) h.cfgsign = cs;
    r.outcome = 4;
  } else {
    for (int i = c.lane; i < K; i += 32) c.opcode[i] = opc_old[i];
    r.outcome = 3;
  }
  __syncwarp();
}

// Accepted tau shift with off-diagonal hybridisation
// (update_InvFullHybrShiftTau_offdiag, Trace.F90:2490-2600): in every
// (creator flavour, annihilator flavour) block the rows and columns rotate
// by the flavour's wrapped creators / annihilators, an entry negated when
// exactly one of its row and column wrapped.  Returns the determinant sign
// change, (-1)^(size x wrapped) per flavour block.  tau_old/opc_old hold
// the operators before the shift (K entries).
__device__ NOINL double shift_od_rotate(Ctx& c, const double* tau_old, const int* opc_old, int K, double dtau) {
  const int nf = c.m->nf, ld = c.kcap, k = K / 2;
  int sz[2 * NFMAX], wr[2 * NFMAX], off[2 * NFMAX];
  for (int q = 0; q < 2 * nf; ++q) {
    int n = 0, w = 0;
    for (int i = c.lane; i < K; i += 32) {
      n += opc_old[i] == q;
      w += opc_old[i] == q && tau_old[i] < dtau;
    }
    sz[q] = wsumi(n);
    wr[q] = wsumi(w);
  }
  double detrat = 1.0;
  for (int q = 0; q < 2 * nf; ++q) {
    off[q] = 0;
    for (int t = q & 1; t < q; t += 2) off[q] += sz[t];
    if ((sz[q] * wr[q]) & 1) detrat = -detrat;
  }
  const double* Mf = M_ptr(c, 0);
  double* T = glob_minv(c);
  for (int e = c.lane; e < k * k; e += 32) {
    const int row = e % k, col = e / k;
    int fr = 0, fc = 0;
    while (fr + 1 < nf && off[2 * (fr + 1)] <= row) ++fr;
    while (fc + 1 < nf && off[2 * (fc + 1) + 1] <= col) ++fc;
    const int qr = 2 * fr, qc = 2 * fc + 1;
    const int i = row - off[qr], j = col - off[qc];
    const int oi = (i + wr[qr]) % sz[qr], oj = (j + wr[qc]) % sz[qc];
    const bool ri = i >= sz[qr] - wr[qr], cj = j >= sz[qc] - wr[qc];
    const double v = Mf[(size_t)(off[qc] + oj) * ld + (off[qr] + oi)];
    T[(size_t)col * ld + row] = ri != cj ? -v : v;
  }
  __syncwarp();
  double* Mw = M_ptr(c, 0);
  for (int e = c.lane; e < k * k; e += 32) {
    const size_t idx = (size_t)(e / k) * ld + (e % k);
    Mw[idx] = T[idx];
  }
  __syncwarp();
  return detrat;
}

// Drift control (no counterpart in the reference, which rebuilds M exactly
// only in global moves and set_mc_config): after every `refresh_every`
// accepted pair updates a chain rebuilds all its inverse matrices by
// Gauss-Jordan elimination from the operator times, records the largest
// deviation of the fast-updated matrices and log-determinant from the
// rebuilt ones, and continues with the rebuilt ones.  The proposal stream is
// unchanged: the rebuild draws no random numbers.
__device__ __forceinline__ bool refresh_due(const Ctx& c) {
  return c.g->refresh_every > 0 && c.h->status == ST_OK && c.h->acc_since_refresh >= c.g->refresh_every;
}
__device__ NOINL void ph_refresh(Ctx& c);

// One proposal of the Z-space loop (CTQMC.F90:8435-8476 / 8212-8250) with
// the phases back to back.
__device__ void one_step(Ctx& c, Prop& p) {
  PROF_START();
  ph_draw(c, p);
  if (p.rare) {
    if (p.move == 2) ph_global(c, p);
    else if (p.move == 3) ph_shift(c, p);
    else if (p.move == 5) ph_add4(c, p);
    else if (p.move == 6) ph_rem4(c, p);
    else if (p.move == 7) ph_add_od(c, p);
    else ph_rem_od(c, p);
    if (refresh_due(c)) ph_refresh(c);
    if (c.h->status == ST_OK) ph_finish(c, p);
    return;
  }
  if (!p.alive) return;  // capacity
  PROF_MARK(0);
  if (p.move == 0) ph_setup_add(c, p);
  else ph_setup_rem(c, p);
  PROF_MARK(1);
  if (p.alive) ph_tree_ss(c, p);
  if (p.alive) ph_tree_states(c, p);
  PROF_MARK(2);
  if (p.alive) ph_det(c, p);
  PROF_MARK(3);
  if (p.alive) ph_trace(c, p);
  if (p.alive) ph_decide(c, p);
  PROF_MARK(4);
  if (p.alive) {
    if (p.move == 0) ph_accept_add(c, p);
    else ph_accept_rem(c, p);
  }
  if (refresh_due(c)) ph_refresh(c);
  PROF_MARK(5);
  if (c.h->status == ST_OK) ph_finish(c, p);
  PROF_MARK(6);
}

// d log|trace| / dtheta_p of the current configuration (monomial models):
// every outer state is walked through the operators; its log weight is
// -sum E(state) * segment, its derivative the same sum with dE_p; the
// derivatives are averaged with the states' signed contributions.  Also
// returns log|trace| (relative to exp(-beta Egs)).  Lane-uniform results.
constexpr int NPARMAX = 32;
__device__ NOINL void trace_score(Ctx& c, const double* __restrict__ dE, int npar, double* score, double& logtr) {
  const DModel& m = *c.m;
  const Hdr& h = *c.h;
  const int s0 = h.outer_sst, off = m.sst_off[s0], n0 = m.sst_n[s0], K = h.K;
  double mx = -DHUGE, S = 0.0, D[NPARMAX];
  for (int p = 0; p < npar; ++p) D[p] = 0.0;
  for (int q = c.lane; q < n0; q += 32) {
    int cur = off + q, neg = 0;
    double l = 0.0, dl[NPARMAX], t = 0.0;
    for (int p = 0; p < npar; ++p) dl[p] = 0.0;
    for (int j = 0; j < K && cur >= 0; ++j) {
      const double tau = c.optau[j], dt = tau - t;
      l -= m.evs[cur] * dt;
      for (int p = 0; p < npar; ++p) dl[p] -= dE[(size_t)p * m.ns + cur] * dt;
      const size_t idx = (size_t)c.opcode[j] * m.ns + cur;
      const int nx = m.mono_tgt[idx];
      if (nx >= 0) {
        l += m.mono_lv[idx];
        neg ^= m.mono_neg[idx];
      }
      cur = nx;
      t = tau;
    }
    if (cur != off + q) continue;
    const double dt = c.g->beta - t;
    l -= m.evs[cur] * dt;
    for (int p = 0; p < npar; ++p) dl[p] -= dE[(size_t)p * m.ns + cur] * dt;
    const double sg = neg ? -1.0 : 1.0;
    if (l > mx) {  // rescale the running sums to the new maximum
      const double r = mx == -DHUGE ? 0.0 : exp(mx - l);
      S *= r;
      for (int p = 0; p < npar; ++p) D[p] *= r;
      mx = l;
    }
    const double w = sg * exp(l - mx);
    S += w;
    for (int p = 0; p < npar; ++p) D[p] += w * dl[p];
  }
  const double gmx = wmax(mx);
  const double r = mx == -DHUGE ? 0.0 : exp(mx - gmx);
  S = wsum(S * r);
  for (int p = 0; p < npar; ++p) score[p] = wsum(D[p] * r) / S;
  logtr = gmx + log(fabs(S));
}

// ---------------------------------------------------------------------------
// Measurements after each NCorr block (CTQMC.F90:8541-8566)
__device__ NOINL void measure(Ctx& c) {
  Hdr& h = *c.h;
  const DModel& m = *c.m;
  const DGroup& g = *c.g;
  if (c.lane == 0) {
    h.cnt_meas++;
    h.meas_sign += h.cfgsign;  // MeasSign
  }
  // MeasExpOrder (off-diagonal groups: in measure_od with G)
  if (g.offdiag) {
    measure_od(c);
  } else {
    for (int f = c.lane; f < m.nf; f += 32) {
      int k = h.k[f];
      int hm = g.maxhisto;
      c.histo[(size_t)f * hm + (k < hm - 1 ? k : hm - 1)] += 1.0;
    }
    __syncwarp();
  }
  // MeasDensityMatrix_beta_half from the two children of the root
  if (g.meas_dm && c.mono) {
    int s0 = h.outer_sst;
    int off = m.sst_off[s0], n0 = m.sst_n[s0];
    const double* lwl = node_lw(c, 2, c.act[2]);
    const uint16_t* tgl = node_tg(c, 2, c.act[2]);
    const double* lwr = node_lw(c, 3, c.act[3]);
    const uint16_t* tgr = node_tg(c, 3, c.act[3]);
    for (int i = c.lane; i < n0; i += 32) {
      int st = off + i;
      uint16_t a = tgl[st];
      int mid = a & 0x7fff;
      if (mid == 0x7fff) continue;
      uint16_t b = tgr[mid];
      if ((b & 0x7fff) != st) continue;
      double sgn = ((a ^ b) & 0x8000) ? -1.0 : 1.0;
      double val = sgn * exp(lwl[st] + lwr[mid] - h.trace_log) * h.trace_sign * (-h.cfgsign);
      c.dm[mid] += val;
    }
    __syncwarp();
  }
  // MeasOuterHistograms (CTQMC.F90:3285-3341, no state sampling); the
  // per-state trace contributions come from the root of the state tree
  {
    const int s0 = h.outer_sst, off = m.sst_off[s0], n0 = m.sst_n[s0];
    double* oh = (double*)((char*)c.gtau - g.o_gtau + g.o_outer);
    // [0,nss) superstate visits, [nss,2nss) superstate signs, [2nss,3nss)
    // superstate contributions, then the same three for states
    double* st_visit = oh + 3 * m.nss;
    double* st_sign = st_visit + m.ns;
    double* st_contr = st_sign + m.ns;
    double csum = 0.0;
    const double* lw = c.mono ? node_lw(c, 1, c.act[1]) : nullptr;
    const uint16_t* tg = c.mono ? node_tg(c, 1, c.act[1]) : nullptr;
    for (int i = c.lane; i < n0; i += 32) {
      const int st = off + i;
      double psign = 1.0, contr = 0.0;
      if (c.mono && (tg[st] & 0x7fff) == st) {
        psign = (tg[st] & 0x8000) ? -1.0 : 1.0;
        contr = exp(lw[st]);
      }
      st_visit[st] += 1.0;
      st_sign[st] += h.trace_sign * psign * h.cfgsign;
      st_contr[st] += contr;
      csum += contr;
    }
    csum = wsum(csum);
    if (c.lane == 0) {
      oh[s0] += 1.0;
      oh[m.nss + s0] += h.cfgsign;
      oh[2 * m.nss + s0] += csum;
    }
    __syncwarp();
  }
  // MeasDensityMatrix_beta_half for dense-block models: kets and bras at the
  // middle edge (beta/2), rho(s1, s2) += bra(s1) ket(s2) / trace per outer
  // state (CTQMC.F90:3088-3150)
  if (g.meas_dm && !c.mono && g.o_chk) {
    const int mid = 1 << (g.L - 1);
    if (ensure_kets(c, mid, solo_team(c)) && ensure_bras(c, mid, solo_team(c))) {
      ChkHead* kh = chk_head(c, 0, mid);
      ChkHead* bh = chk_head(c, 1, mid);
      if (kh->sst == bh->sst) {
        const int sst = kh->sst, n = kh->rows, cols = kh->cols, ld = m.nsmax;
        const double* kv = chk_v(c, kh);
        const double* bv = chk_v(c, bh);
        const double* klg = chk_lg(kh);
        const double* blg = chk_lg(bh);
        double* D = c.dm + m.dm_off[sst];
        const double sgn = h.trace_sign * (-h.cfgsign);
        double* wcol = dwork(c, 3);  // per-column weight, one exponential each
        for (int col = c.lane; col < cols; col += 32) wcol[col] = exp(klg[col] + blg[col] - h.trace_log);
        __syncwarp();
        for (int e = c.lane; e < n * n; e += 32) {
          const int s1 = e % n, s2 = e / n;
          double acc = 0.0;
          for (int col = 0; col < cols; ++col) acc += bv[(size_t)col * ld + s1] * kv[(size_t)col * ld + s2] * wcol[col];
          D[(size_t)s2 * n + s1] += acc * sgn;
        }
        __syncwarp();
      }
    }
  }
  // score-function dG/dtheta: d log|trace| / dtheta of this configuration
  const int nsc = g.nscore;
  double score[NPARMAX];
  double* sacc = nsc > 0 ? (double*)((char*)c.gtau - g.o_gtau + g.o_score) : nullptr;
  if (nsc > 0) {
    double ltr;
    trace_score(c, g.score_dE, nsc, score, ltr);
    if (c.lane == 0)
      for (int p = 0; p < nsc; ++p) sacc[p] += score[p];
    __syncwarp();
  }
  // MeasGtauRem(.false.): M elements binned by tau_a - tau_c, and their
  // Legendre coefficients (CTQMC.F90:2252-2440)
  const int nt = g.ntau, nleg = g.nleg;
  double* lsum = nleg > 0 ? (double*)((char*)c.gtau - g.o_gtau + g.o_glscr) + (size_t)c.lane * nleg : nullptr;
  for (int f = 0; f < m.nf; ++f) {
    int k = h.k[f];
    const double* Mf = M_ptr(c, f);
    const double* tcs = stau_ptr(c, f, 0);
    const double* tas = stau_ptr(c, f, 1);
    double* G = c.gtau + (size_t)f * nt;
    for (int l = 0; l < nleg; ++l) lsum[l] = 0.0;
    for (int i = c.lane; i < k; i += 32) {
      double tc = tcs[i];
      for (int j = 0; j < k; ++j) {
        double Mv = Mf[(size_t)j * c.kcap + i];
        double ta = tas[j];
        double dt;
        if (ta - tc > 0.0) {
          dt = ta - tc;
        } else {
          dt = g.beta + ta - tc;
          Mv = -Mv;
        }
        // idt = int(dt / beta * Ntau) + 1, evaluated exactly as written
        // where dt * (Ntau / beta) lies close to a bin edge
        const double q = dt * g.gscale;
        int idt = (int)q;
        const double fr = q - (double)idt;
        if (fr < 1e-9 || fr > 1.0 - 1e-9) idt = (int)__dmul_rn(__ddiv_rn(dt, g.beta), (double)nt);
        idt += 1;
        Mv = Mv * h.cfgsign;
        if (idt > nt) idt = nt;
        atomicAdd(&G[idt - 1], Mv);
        for (int p = 0; p < nsc; ++p) atomicAdd(&sacc[nsc + ((size_t)p * m.nf + f) * nt + idt - 1], Mv * score[p]);
        if (nleg > 0) legendre_add(Mv, __dsub_rn(__dmul_rn(__ddiv_rn(2.0, g.beta), dt), 1.0), nleg, lsum);
      }
    }
    if (nleg > 0) {
      __syncwarp();
      double* GL = (double*)((char*)c.gtau - g.o_gtau + g.o_gleg) + (size_t)f * nleg;
      for (int l = 0; l < nleg; ++l) {
        const double v = wsum(lsum[l]);
        if (c.lane == 0) GL[l] += v;
      }
      __syncwarp();
    }
  }
  __syncwarp();
}

// ---------------------------------------------------------------------------
// Kernels
__device__ Ctx make_ctx(const DModel* m, const DGroup* g, Hdr* hsm, int chain, cthyb_record* rec = nullptr) {
  Ctx c;
  c.rec = rec;
  c.m = m;
  c.g = g;
  c.h = hsm;
  c.lane = threadIdx.x & 31;
  c.chain = chain;
  char* b = g->base + (size_t)chain * g->stride;
  c.mt = (uint32_t*)(b + g->o_mt);
  c.optau = (double*)(b + g->o_optau);
  c.opcode = (int*)(b + g->o_opcode);
  c.srt_tau = (double*)(b + g->o_srt_tau);
  c.srt_slot = (short*)(b + g->o_srt_slot);
  c.slot_tau = (double*)(b + g->o_slot_tau);
  c.M = (double*)(b + g->o_M);
  c.tree = b + g->o_tree;
  c.act = (unsigned char*)(b + g->o_act);
  c.bstart = (int*)(b + g->o_bstart);
  c.scr = (double*)(b + g->o_scr);
  c.btau[0] = c.scr + 4 * g->kcap;
  c.btau[1] = c.btau[0] + g->opcap + 2;
  c.bdt[0] = c.btau[1] + g->opcap + 2;
  c.bdt[1] = c.bdt[0] + g->opcap + 3;
  c.bcode[0] = (int*)(c.bdt[1] + g->opcap + 3);
  c.bcode[1] = c.bcode[0] + g->opcap + 2;
  c.gtau = (double*)(b + g->o_gtau);
  c.histo = (double*)(b + g->o_histo);
  c.dm = (double*)(b + g->o_dm);
  c.dense = (double*)(b + g->o_dense);
  c.log = g->logcap > 0 ? (cthyb_record*)(b + g->o_log) : nullptr;
  c.kcap = g->kcap;
  c.mono = m->monomial && !g->dense;
  return c;
}

constexpr int WPB = 4;  // warps (chains) per block
#ifndef SWEEP_MIN_BLOCKS
#define SWEEP_MIN_BLOCKS 8  // resident blocks per SM the register budget aims for
#endif

__device__ __forceinline__ void load_hdr(Hdr* dst, const Hdr* src, int lane) {
  const int n = sizeof(Hdr) / 4;
  for (int i = lane; i < n; i += 32) ((int*)dst)[i] = ((const int*)src)[i];
  __syncwarp();
}
__device__ __forceinline__ void store_hdr(Hdr* dst, const Hdr* src, int lane) {
  __syncwarp();
  const int n = sizeof(Hdr) / 4;
  for (int i = lane; i < n; i += 32) ((int*)dst)[i] = ((const int*)src)[i];
  __syncwarp();
}

// init_Trace (Trace.F90:340-701) for every chain of a group.
__global__ void __launch_bounds__(WPB * 32) k_init(const __grid_constant__ DModel m, const __grid_constant__ DGroup g,
                                                  const int* seeds, const double* tdm, int ncorr) {
  __shared__ Hdr hs[WPB];
  int warp = threadIdx.x >> 5;
  int chain = blockIdx.x * WPB + warp;
  if (chain >= g.nchains) return;
  Ctx c = make_ctx(&m, &g, &hs[warp], chain);
  Hdr& h = *c.h;
  if (c.lane == 0) {
    memset(&h, 0, sizeof(Hdr));
    h.det_log = 0.0;
    h.det_sign = 1.0;
    h.cfgsign = -1.0;
    h.trace_sign = 1.0;
  }
  __syncwarp();
  mt_seed(c.mt, (uint32_t)seeds[chain], c.lane);
  mt_refill(c, 624);
  init_window(c, *tdm);
  if (c.lane == 0) {
    h.npairs = 0;
    int nsl = (int)floor((double)ncorr / (double)h.num_windows);
    h.nslide = nsl > 2 * m.nd ? nsl : 2 * m.nd;
  }
  __syncwarp();
  // outer superstate in proportion to the empty trace
  double rnd = grnd(c);
  if (c.lane == 0) {
    double acc = 0.0;
    for (int s = 0; s < m.nss; ++s) {
      h.outer_sst = s;
      acc += g.empty_w[s];
      if (acc >= rnd && g.empty_w[s] != 0.0) break;
    }
  }
  __syncwarp();
  // empty configuration
  if (c.lane == 0) h.K = 0;
  __syncwarp();
  tree_build_all(c);
  chk_invalidate(c);
  double lg, sg;
  if (c.mono) {
    double mx, sum;
    root_trace(c, 0, h.outer_sst, mx, sum);
    trace_log(mx, sum, lg, sg);
  } else {
    Mod md;
    md.type = 0;
    dense_trace(c, md, h.outer_sst, lg, sg, solo_team(c));
  }
  if (c.lane == 0) {
    h.trace_log = lg;
    h.trace_sign = sg;
    h.mt_idx = mt_index(c);
  }
  store_hdr((Hdr*)(g.base + (size_t)chain * g.stride + g.o_hdr), &h, c.lane);
}

// One launch advances every chain of every group: warp -> (group, chain).
__global__ void __launch_bounds__(WPB * 32, SWEEP_MIN_BLOCKS)
    k_sweep(const __grid_constant__ DModel m, const DGroup* __restrict__ groups, int ngroups, int ntotal,
            long long nprop, int nmeas, int reset, int actbytes) {
  __shared__ Hdr hs[WPB];
  __shared__ cthyb_record recs[WPB];
  __shared__ Prop props[WPB];
  extern __shared__ __align__(16) unsigned char dyn_act[];
  int warp = threadIdx.x >> 5;
  int gchain = blockIdx.x * WPB + warp;
  if (gchain >= ntotal) return;
  int gi = 0;
  while (gi + 1 < ngroups && gchain >= groups[gi + 1].chain0) ++gi;
  const DGroup& g = groups[gi];
  int chain = gchain - g.chain0;
  Ctx c = make_ctx(&m, &g, &hs[warp], chain, &recs[warp]);
  Hdr* gh = (Hdr*)(g.base + (size_t)chain * g.stride + g.o_hdr);
  load_hdr(c.h, gh, c.lane);
  // the tree's active bits live in shared memory during the sweep
  unsigned char* gact = c.act;
  const int nact4 = ((2 << g.L) + 3) / 4;  // whole words (a one-leaf tree has 2 bytes)
  c.act = dyn_act + (size_t)warp * actbytes;
  for (int i = c.lane; i < nact4; i += 32) ((uint32_t*)c.act)[i] = ((const uint32_t*)gact)[i];
  __syncwarp();
  Hdr& h = *c.h;
  mt_refill(c, h.mt_idx);
  if (reset && c.lane == 0) {  // init_counters, CTQMC.F90:847-899
    h.try_add = h.acc_add = h.try_rem = h.acc_rem = h.qn_add = h.qn_rem = 0;
    h.try_glob = h.acc_glob = h.qn_glob = h.try_shift = h.acc_shift = 0;
    h.try_add4 = h.acc_add4 = h.try_rem4 = h.acc_rem4 = 0;
    h.nprop = 0;
  }
  __syncwarp();
  if (h.status == ST_OK) {
    if (nmeas <= 0) {
      for (long long i = 0; i < nprop && h.status == ST_OK; ++i) one_step(c, props[warp]);
    } else {
      for (int im = 0; im < nmeas && h.status == ST_OK; ++im) {
        for (int ic = 0; ic < g.ncorr && h.status == ST_OK; ++ic) one_step(c, props[warp]);
        PROF_START();
        if (h.status == ST_OK) measure(c);
        PROF_MARK(9);
      }
    }
  }
  if (c.lane == 0) {
    h.mt_idx = mt_index(c);
    if (h.status != ST_OK) atomicMax(g.err_flag, h.status);
  }
  __syncwarp();
  for (int i = c.lane; i < nact4; i += 32) ((uint32_t*)gact)[i] = ((const uint32_t*)c.act)[i];
  store_hdr(gh, c.h, c.lane);
}

// Phase-synchronous sweep: the warps of a block (one chain each) run the
// phases of their proposals together, with a block-wide barrier between
// phases, so that the SM's instruction caches serve the code of one phase at
// a time instead of every warp's own position in the proposal.  Per-warp
// header, record, proposal state and tree active bits live in dynamic shared
// memory.  Results are those of k_sweep: each chain's proposal sequence is
// unchanged, only the interleaving of chains differs.
#ifndef SYNC_MAX_THREADS
#define SYNC_MAX_THREADS 1024  // register budget: 64 per thread, 32 chain warps per SM
#define SYNC_MIN_BLOCKS 1
#endif
// Shared-memory residence of one chain (blocks of one chain warp): three
// contiguous ranges of the chain's slab -- operator arrays and sorted lists
// [o_optau, o_M), the time-bin tree [o_tree, o_act), bin starts and scratch
// [o_bstart, o_gtau) -- are copied into the block's shared memory and the
// context's pointers redirected there; on leaving, the ranges go back.  The
// inverse matrices, accumulators, checkpoints and rare-move space stay in
// global memory.  Every access to these ranges in the sweep goes through
// the context's pointers.
__host__ __device__ inline size_t resident_bytes(const DGroup& g) {
  return (g.o_M - g.o_optau) + (g.o_act - g.o_tree) + (g.o_gtau - g.o_bstart);
}
__device__ __forceinline__ void copy16(void* dst, const void* src, size_t bytes, int lane) {
  uint4* d = (uint4*)dst;
  const uint4* sp = (const uint4*)src;
  for (size_t i = lane; i < bytes / 16; i += 32) d[i] = sp[i];
}
__device__ NOINL void resident_enter(Ctx& c, unsigned char* sm) {
  const DGroup& g = *c.g;
  const char* b = g.base + (size_t)c.chain * g.stride;
  const size_t la = g.o_M - g.o_optau, lt = g.o_act - g.o_tree, ls = g.o_gtau - g.o_bstart;
  char* sa = (char*)sm;
  char* st = sa + la;
  char* ss = st + lt;
  copy16(sa, b + g.o_optau, la, c.lane);
  copy16(st, b + g.o_tree, lt, c.lane);
  copy16(ss, b + g.o_bstart, ls, c.lane);
  __syncwarp();
  c.optau = (double*)(sa);
  c.opcode = (int*)(sa + (g.o_opcode - g.o_optau));
  c.srt_tau = (double*)(sa + (g.o_srt_tau - g.o_optau));
  c.srt_slot = (short*)(sa + (g.o_srt_slot - g.o_optau));
  c.slot_tau = (double*)(sa + (g.o_slot_tau - g.o_optau));
  c.tree = st;
  c.bstart = (int*)ss;
  c.scr = (double*)(ss + (g.o_scr - g.o_bstart));
  c.btau[0] = c.scr + 4 * g.kcap;
  c.btau[1] = c.btau[0] + g.opcap + 2;
  c.bdt[0] = c.btau[1] + g.opcap + 2;
  c.bdt[1] = c.bdt[0] + g.opcap + 3;
  c.bcode[0] = (int*)(c.bdt[1] + g.opcap + 3);
  c.bcode[1] = c.bcode[0] + g.opcap + 2;
}
__device__ NOINL void resident_leave(Ctx& c, const unsigned char* sm) {
  const DGroup& g = *c.g;
  char* b = g.base + (size_t)c.chain * g.stride;
  const size_t la = g.o_M - g.o_optau, lt = g.o_act - g.o_tree;
  const char* sa = (const char*)sm;
  copy16(b + g.o_optau, sa, la, c.lane);
  copy16(b + g.o_tree, sa + la, lt, c.lane);
  copy16(b + g.o_bstart, sa + la + lt, g.o_gtau - g.o_bstart, c.lane);
  __syncwarp();
}

__global__ void __launch_bounds__(SYNC_MAX_THREADS, SYNC_MIN_BLOCKS)
    k_sweep_sync(const __grid_constant__ DModel m, const DGroup* __restrict__ groups, int ngroups, int ntotal,
                 long long nprop, int nmeas, int reset, int actbytes, int resident_off) {
  extern __shared__ __align__(16) unsigned char dyn[];
  const int nw = blockDim.x >> 5, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  Hdr* hs = (Hdr*)dyn;
  cthyb_record* recs = (cthyb_record*)(hs + nw);
  Prop* props = (Prop*)(recs + nw);
  unsigned char* acts = (unsigned char*)(props + nw);
  const int gchain = blockIdx.x * nw + warp;
  const bool valid = gchain < ntotal;
  Prop& p = props[warp];
  Ctx c;
  const DGroup* gp = nullptr;
  unsigned char* gact = nullptr;
  Hdr* gh = nullptr;
  long long total = 0;
  int nact4 = 0;
  if (valid) {
    int gi = 0;
    while (gi + 1 < ngroups && gchain >= groups[gi + 1].chain0) ++gi;
    gp = &groups[gi];
    const int chain = gchain - gp->chain0;
    c = make_ctx(&m, gp, &hs[warp], chain, &recs[warp]);
    gh = (Hdr*)(gp->base + (size_t)chain * gp->stride + gp->o_hdr);
    load_hdr(c.h, gh, lane);
    gact = c.act;
    nact4 = ((2 << gp->L) + 3) / 4;
    c.act = acts + (size_t)warp * actbytes;
    for (int i = lane; i < nact4; i += 32) ((uint32_t*)c.act)[i] = ((const uint32_t*)gact)[i];
    __syncwarp();
    if (resident_off) resident_enter(c, dyn + resident_off);
    mt_refill(c, c.h->mt_idx);
    if (reset && lane == 0) {  // init_counters, CTQMC.F90:847-899
      Hdr& h = *c.h;
      h.try_add = h.acc_add = h.try_rem = h.acc_rem = h.qn_add = h.qn_rem = 0;
      h.try_glob = h.acc_glob = h.qn_glob = h.try_shift = h.acc_shift = 0;
      h.try_add4 = h.acc_add4 = h.try_rem4 = h.acc_rem4 = 0;
      h.nprop = 0;
    }
    __syncwarp();
    total = nmeas <= 0 ? nprop : (long long)nmeas * gp->ncorr;
  }
  // One barrier after each phase: set-up, superstate tree + QN check, state
  // tree, determinant, trace, decision with the accepted move's updates,
  // rare moves (only when one is pending), and bookkeeping + measurement +
  // the next draw.  A warp with nothing to do in a phase (proposal ended,
  // chain finished, no chain) only meets the barrier.
  long long i = 0;
#ifdef CTHYB_PROFILE
  // prof[k]: work of phase k (0..8, phase 8 = bookkeeping); prof[9]: waits
#define SPROF(k)  \
  if (valid) {    \
    PROF_MARK(k); \
  }
  PROF_START();
#else
#define SPROF(k)
#endif
#define PHASE(k, stmt) \
  if (p.alive) {       \
    stmt;              \
  }                    \
  SPROF(k);            \
  __syncthreads();     \
  SPROF(9);
  // the next proposal's draw shares the segment of the previous one's
  // bookkeeping; the barrier that follows also decides whether any chain of
  // the block is left
  bool mine = valid && i < total && c.h->status == ST_OK;
  if (mine) {
    ph_draw(c, p);
  } else if (lane == 0) {
    p.alive = 0;
    p.rare = 0;
  }
  SPROF(0);
  while (__syncthreads_or(mine)) {
    SPROF(9);
    PHASE(1, if (p.move == 0) ph_setup_add(c, p); else ph_setup_rem(c, p))
    PHASE(2, ph_tree_ss(c, p))
    PHASE(3, ph_tree_states(c, p))
    PHASE(4, ph_det(c, p))
    PHASE(5, ph_trace(c, p))
    if (p.alive) {
      ph_decide(c, p);
      if (p.alive) {
        if (p.move == 0) ph_accept_add(c, p);
        else ph_accept_rem(c, p);
      }
    }
    SPROF(6);
    // rare moves and the periodic rebuilds of M share one optional phase
    if (__syncthreads_or(p.rare || (mine && refresh_due(c)))) {
      if (p.rare) {
        if (p.move == 2) ph_global(c, p);
        else if (p.move == 3) ph_shift(c, p);
        else if (p.move == 5) ph_add4(c, p);
        else if (p.move == 6) ph_rem4(c, p);
        else if (p.move == 7) ph_add_od(c, p);
        else ph_rem_od(c, p);
      }
      if (mine && refresh_due(c)) ph_refresh(c);
      __syncthreads();
    }
    if (mine && c.h->status == ST_OK) {
      ph_finish(c, p);
      ++i;
      if (nmeas > 0 && i % gp->ncorr == 0 && c.h->status == ST_OK) measure(c);
    }
    SPROF(8);
    mine = valid && i < total && c.h->status == ST_OK;
    if (mine) {
      ph_draw(c, p);
    } else if (lane == 0) {
      p.alive = 0;
      p.rare = 0;
    }
    SPROF(0);
  }
#undef PHASE
#undef SPROF
  if (valid) {
    if (lane == 0) {
      c.h->mt_idx = mt_index(c);
      if (c.h->status != ST_OK) atomicMax(gp->err_flag, c.h->status);
    }
    __syncwarp();
    if (resident_off) resident_leave(c, dyn + resident_off);
    for (int i2 = lane; i2 < nact4; i2 += 32) ((uint32_t*)gact)[i2] = ((const uint32_t*)c.act)[i2];
    store_hdr(gh, c.h, lane);
  }
}

// Team sweep: each block is a team of T warps that advances one chain at a
// time; chains are taken in the order of `order` through a global counter,
// so a block that finishes early picks up the next chain (the order puts
// the largest estimated cost first: longest-processing-time-first list
// scheduling over the blocks).  Warp 0 runs the scalar phases of every
// proposal with the same functions as the other sweeps, so each chain's
// proposal stream is unchanged; the whole team evaluates the dense-block
// trace (block products, renormalisation, checkpoints).
#ifndef TEAM_MAX_THREADS
#define TEAM_MAX_THREADS 512  // teams of up to 16 warps
#define TEAM_MIN_BLOCKS 2     // register budget: 64 per thread
#endif
__global__ void __launch_bounds__(TEAM_MAX_THREADS, TEAM_MIN_BLOCKS)
    k_sweep_team(const __grid_constant__ DModel m, const DGroup* __restrict__ groups, int ngroups, int ntotal,
                 long long nprop, int nmeas, int reset, const int* __restrict__ order, int* counter) {
  extern __shared__ __align__(16) unsigned char dyn[];
  Hdr* hs = (Hdr*)dyn;
  cthyb_record* rec = (cthyb_record*)(hs + 1);
  Prop* pp = (Prop*)(rec + 1);
  double* red = (double*)(pp + 1);                   // one double per warp
  unsigned char* act = (unsigned char*)(red + 32);   // tree active bits
  __shared__ int next;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const Team team{(int)threadIdx.x, (int)blockDim.x, red};
  Prop& p = *pp;
  while (true) {
    if (threadIdx.x == 0) next = atomicAdd(counter, 1);
    __syncthreads();
    const int slot = next;
    __syncthreads();
    if (slot >= ntotal) break;
    const int gchain = order[slot];
    int gi = 0;
    while (gi + 1 < ngroups && gchain >= groups[gi + 1].chain0) ++gi;
    const DGroup* gp = &groups[gi];
    const int chain = gchain - gp->chain0;
    Ctx c = make_ctx(&m, gp, hs, chain, rec);
    Hdr* gh = (Hdr*)(gp->base + (size_t)chain * gp->stride + gp->o_hdr);
    unsigned char* gact = c.act;
    const int nact4 = ((2 << gp->L) + 3) / 4;
    c.act = act;
    if (warp == 0) {
      load_hdr(c.h, gh, lane);
      for (int i = lane; i < nact4; i += 32) ((uint32_t*)c.act)[i] = ((const uint32_t*)gact)[i];
      __syncwarp();
      mt_refill(c, c.h->mt_idx);
      if (reset && lane == 0) {  // init_counters, CTQMC.F90:847-899
        Hdr& h = *c.h;
        h.try_add = h.acc_add = h.try_rem = h.acc_rem = h.qn_add = h.qn_rem = 0;
        h.try_glob = h.acc_glob = h.qn_glob = h.try_shift = h.acc_shift = 0;
        h.try_add4 = h.acc_add4 = h.try_rem4 = h.acc_rem4 = 0;
        h.nprop = 0;
      }
      __syncwarp();
    }
    __syncthreads();
    const long long total = nmeas <= 0 ? nprop : (long long)nmeas * gp->ncorr;
    for (long long i = 0; i < total; ++i) {
      if (c.h->status != ST_OK) break;  // the shared header, read after a block barrier
      if (warp == 0) {
        ph_draw(c, p);
        if (p.rare) {
          if (p.move == 2) ph_global(c, p);
          else if (p.move == 3) ph_shift(c, p);
          else if (p.move == 5) ph_add4(c, p);
          else if (p.move == 6) ph_rem4(c, p);
          else if (p.move == 7) ph_add_od(c, p);
          else ph_rem_od(c, p);
          if (refresh_due(c)) ph_refresh(c);
          if (c.h->status == ST_OK) ph_finish(c, p);
        } else if (p.alive) {
          if (p.move == 0) ph_setup_add(c, p);
          else ph_setup_rem(c, p);
          if (p.alive) ph_tree_ss(c, p);
          if (p.alive) ph_tree_states(c, p);
          if (p.alive) ph_det(c, p);
        }
      }
      __syncthreads();
      if (!p.rare && p.alive) ph_trace_team(c, p, team);  // the whole team; ends with a barrier
      if (warp == 0) {
        if (!p.rare) {
          if (p.alive) ph_decide(c, p);
          if (p.alive) {
            if (p.move == 0) ph_accept_add(c, p);
            else ph_accept_rem(c, p);
          }
          if (refresh_due(c)) ph_refresh(c);
          if (c.h->status == ST_OK) ph_finish(c, p);
        }
      }
      if (nmeas > 0 && (i + 1) % gp->ncorr == 0) {
        // dense-block models: the team extends the checkpoints to the
        // middle edge first, so the density-matrix measurement at beta/2
        // finds them valid
        __syncthreads();
        if (gp->meas_dm && !c.mono && gp->o_chk && c.h->status == ST_OK) {
          const int mid = 1 << (gp->L - 1);
          if (ensure_kets(c, mid, team)) ensure_bras(c, mid, team);
        }
        if (warp == 0 && c.h->status == ST_OK) measure(c);
      }
      __syncthreads();
    }
    if (warp == 0) {
      if (lane == 0) {
        c.h->mt_idx = mt_index(c);
        if (c.h->status != ST_OK) atomicMax(gp->err_flag, c.h->status);
      }
      __syncwarp();
      for (int i2 = lane; i2 < nact4; i2 += 32) ((uint32_t*)gact)[i2] = ((const uint32_t*)c.act)[i2];
      store_hdr(gh, c.h, lane);
    }
    __syncthreads();
  }
}

// Order of the chains for the team sweep: estimated cost of a proposal
// descending (operators + 8, times the outer superstate's size for dense-
// block models: the trace's block products scale with both), ties by
// chain index; one block, bitonic sort of (cost, index) keys in shared
// memory for up to 8192 chains, the identity beyond.
constexpr int ORDER_MAX = 8192;
__global__ void __launch_bounds__(1024) k_order(const __grid_constant__ DModel m, const DGroup* __restrict__ groups,
                                                int ngroups, int ntotal, int* __restrict__ order) {
  extern __shared__ unsigned long long keys[];
  int n2 = 1;
  while (n2 < ntotal) n2 <<= 1;
  if (n2 > ORDER_MAX) {
    for (int i = threadIdx.x; i < ntotal; i += blockDim.x) order[i] = i;
    return;
  }
  for (int i = threadIdx.x; i < n2; i += blockDim.x) {
    unsigned long long v = ~0ull;
    if (i < ntotal) {
      int gi = 0;
      while (gi + 1 < ngroups && i >= groups[gi + 1].chain0) ++gi;
      const DGroup& g = groups[gi];
      const Hdr* h = (const Hdr*)(g.base + (size_t)(i - g.chain0) * g.stride + g.o_hdr);
      long long cost = (long long)h->K + 8;
      if (!(m.monomial && !g.dense)) cost *= m.sst_n[h->outer_sst];
      const long long key = cost < 0x7fffffffll ? cost : 0x7fffffffll;
      v = ((unsigned long long)(0x7fffffffll - key) << 32) | (unsigned)i;
    }
    keys[i] = v;
  }
  __syncthreads();
  for (int k = 2; k <= n2; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < n2; i += blockDim.x) {
        const int ixj = i ^ j;
        if (ixj > i) {
          const bool up = (i & k) == 0;
          const unsigned long long a = keys[i], b = keys[ixj];
          if ((a > b) == up) {
            keys[i] = b;
            keys[ixj] = a;
          }
        }
      }
      __syncthreads();
    }
  for (int i = threadIdx.x; i < ntotal; i += blockDim.x) order[i] = (int)(keys[i] & 0xffffffffull);
}

// Gradients of log|w| of each chain's current configuration (no reference
// counterpart).  Determinant part: d log|det H| / dH(a, c) = M(c, a), and
// H(a, c) = Delta_f(tau_a - tau_c) interpolates the grid linearly
// (get_HybrF, Trace.F90:1014-1033), so M(c, a) * sign * (1 - frac) goes to
// grid point i and M(c, a) * sign * frac to i + 1.  Trace part (monomial
// models): each surviving outer state's log weight is minus the sum over
// segments of E(state) * length; along a parameter direction with per-state
// energy derivatives dE it changes by the same sum with dE, and d log|tr| is
// the average of those over the states weighted by their signed
// contributions.  One warp per chain; the walk is O(K) per state.
__global__ void __launch_bounds__(WPB * 32) k_grad(const __grid_constant__ DModel m, const __grid_constant__ DGroup g,
                                                  const double* __restrict__ dE, int npar, double* gdelta,
                                                  double* gpar, double* logw) {
  __shared__ Hdr hs[WPB];
  const int warp = threadIdx.x >> 5;
  const int chain = blockIdx.x * WPB + warp;
  if (chain >= g.nchains) return;
  Ctx c = make_ctx(&m, &g, &hs[warp], chain);
  load_hdr(c.h, (Hdr*)(g.base + (size_t)chain * g.stride + g.o_hdr), c.lane);
  Hdr& h = *c.h;
  const int nft = g.nftau;
  double* gd = gdelta + (size_t)chain * m.nf * nft;
  for (int f = 0; f < m.nf; ++f) {
    const int k = h.k[f];
    const double* Mf = M_ptr(c, f);
    const double* tcs = stau_ptr(c, f, 0);
    const double* tas = stau_ptr(c, f, 1);
    for (int e = c.lane; e < k * k; e += 32) {
      const int sc = e % k, sa = e / k;
      const double Mv = Mf[(size_t)sa * c.kcap + sc];
      double dt = tas[sa] - tcs[sc], sig = 1.0;
      if (dt < 0.0) {
        dt = dt + g.beta;
        sig = -1.0;
      }
      const double n = dt / g.beta * (double)(nft - 1);
      int i = (int)n;
      const double fr = n - (double)(int)n;
      if (i > nft - 2) i = nft - 2;
      atomicAdd(&gd[(size_t)f * nft + i], Mv * sig * (1.0 - fr));
      atomicAdd(&gd[(size_t)f * nft + i + 1], Mv * sig * fr);
    }
  }
  __syncwarp();
  if (c.lane == 0) logw[2 * (size_t)chain] = h.det_log;
  if (!c.mono || npar <= 0) return;
  double score[NPARMAX], ltr;
  trace_score(c, dE, npar, score, ltr);
  if (c.lane == 0)
    for (int p = 0; p < npar; ++p) gpar[(size_t)chain * npar + p] = score[p];
  // absolute log|trace| (the stored trace is relative to exp(-beta Egs))
  if (c.lane == 0) logw[2 * (size_t)chain + 1] = ltr - g.beta * m.egs;
}

// Trace gradients of dense-block models along Hamiltonian directions
// dH/dtheta_p, given as blocks V_p in the eigenbasis of each superstate:
// d log|Tr| / dtheta_p = (1/Tr) sum over the segments between operators of
// Tr[bra_seg^T dP_seg ket_seg], with dP(a, b) = -V_p(a, b) psi(E_a, E_b)
// the exact derivative of the segment propagator exp(-dtau H) in its
// eigenbasis (psi = (exp(-dtau E_a) - exp(-dtau E_b)) / (E_b - E_a), dtau
// exp(-dtau E_a) for E_a = E_b; no eigenvector derivatives are needed,
// the trace being basis-independent).  The adjoint sweep recomputes from
// the checkpoints: per time bin the kets after each operator are stored
// (forward from the ket checkpoint at the bin's start) and the bra is
// propagated backwards from the bra checkpoint at its end.  One block (a
// team of warps) per chain; `scr` holds maxseg + 1 matrices per chain.
__global__ void __launch_bounds__(128) k_grad_dense(const __grid_constant__ DModel m, const __grid_constant__ DGroup g,
                                                    int chain0, const double* __restrict__ vblk, int npar,
                                                    double* gpar, double* logw, double* scr, size_t scr_stride,
                                                    int maxseg) {
  __shared__ Hdr hs;
  __shared__ double red[4];
  const int chain = chain0 + blockIdx.x;
  if (chain >= g.nchains) return;
  const Team t{(int)threadIdx.x, (int)blockDim.x, red};
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  Ctx c = make_ctx(&m, &g, &hs, chain);
  Hdr* gh = (Hdr*)(g.base + (size_t)chain * g.stride + g.o_hdr);
  if (warp == 0) load_hdr(c.h, gh, lane);
  __syncthreads();
  const int nb = 1 << g.L, ld = m.nsmax;
  double* S = scr + (size_t)blockIdx.x * scr_stride;  // stored kets (maxseg + 1) x nsmax^2, then their logs
  double* Slg = S + (size_t)(maxseg + 1) * ld * ld;
  int* Ssst = (int*)(Slg + (size_t)(maxseg + 1) * ld);
  double acc[NPARMAX];
  for (int q = 0; q < npar; ++q) acc[q] = 0.0;
  bool ok = ensure_kets(c, nb, t) && ensure_bras(c, 0, t);
  double trlg = -DHUGE, trsg = 0.0;
  if (ok) {
    // the trace at beta: the full ket against the identity bra
    double *v = dwork(c, 0), *lg = dwork(c, 2);
    int sst, rows, cols;
    chk_load(c, chk_head(c, 0, nb), sst, rows, cols, v, lg, t);
    chk_close(c, sst, rows, cols, v, lg, chk_head(c, 1, nb), trlg, trsg, t);
    ok = trsg != 0.0;
  }
  for (int b = 0; b < nb && ok; ++b) {
    const int j0 = c.bstart[b], nops = c.bstart[b + 1] - j0;
    if (nops > maxseg) {
      ok = false;
      break;
    }
    // forward: S[0] = ket at edge b, S[j] = ket after the j-th operator of the bin
    double *v = dwork(c, 0), *o = dwork(c, 1), *lg = dwork(c, 2);
    int sst, rows, cols;
    chk_load(c, chk_head(c, 0, b), sst, rows, cols, v, lg, t);
    double tt = bin_edge(c, b);
    for (int j = 0; j <= nops; ++j) {
      double* Sj = S + (size_t)j * ld * ld;
      for (int e = t.tid; e < rows * cols; e += t.nth) {
        const size_t x = (size_t)(e / rows) * ld + e % rows;
        Sj[x] = v[x];
      }
      for (int col = t.tid; col < cols; col += t.nth) Slg[(size_t)j * ld + col] = lg[col];
      if (t.tid == 0) Ssst[j] = sst;
      tsync(t);
      if (j == nops) break;
      const double tau = c.optau[j0 + j];
      if (!col_step(c, sst, rows, cols, v, o, lg, c.opcode[j0 + j], false, tau - tt, t)) {
        ok = false;
        break;
      }
      tt = tau;
    }
    if (!ok) break;
    // backward: the bra at the end of each segment, from the checkpoint at edge b + 1
    int bsst, brows, bcols;
    chk_load(c, chk_head(c, 1, b + 1), bsst, brows, bcols, v, lg, t);
    for (int j = nops; j >= 0 && ok; --j) {
      const double ta = j == 0 ? bin_edge(c, b) : c.optau[j0 + j - 1];
      const double te = j == nops ? bin_edge(c, b + 1) : c.optau[j0 + j];
      const double dt = te - ta;
      const int s = Ssst[j];
      if (s != bsst) {
        ok = false;
        break;
      }
      const int n = m.sst_n[s];
      const double* E = m.eval + m.sst_off[s];
      const double e0 = E[0];
      const double* Sj = S + (size_t)j * ld * ld;
      const double* Sl = Slg + (size_t)j * ld;
      double* w = dwork(c, 3);  // per-column weight exp(log ket + log bra - (e0 - Egs) dt - log Tr)
      for (int col = t.tid; col < cols; col += t.nth) w[col] = exp(Sl[col] + lg[col] - (e0 - m.egs) * dt - trlg);
      tsync(t);
      // sum over (b, a) of W(b, a) psi(a, b) (-V_p(a, b)), W = ket w bra^T
      for (int e = t.tid; e < n * n; e += t.nth) {
        const int ib = e % n, ia = e / n;
        double wba = 0.0;
        for (int col = 0; col < cols; ++col) wba = fma(Sj[(size_t)col * ld + ib] * w[col], v[(size_t)col * ld + ia], wba);
        const double d = E[ib] - E[ia];
        const double ea = exp(-(E[ia] - e0) * dt);
        const double psi = d == 0.0 ? dt * ea : ea * (-expm1(-dt * d)) / d;
        const double x = wba * psi;
        for (int q = 0; q < npar; ++q) acc[q] -= vblk[(size_t)q * m.dm_size + m.dm_off[s] + (size_t)ib * n + ia] * x;
      }
      tsync(t);  // the bra and the weights are read above and overwritten below
      if (j == 0) break;
      // bra across segment j and through the j-th operator (transposed)
      if (!col_step(c, bsst, brows, bcols, v, o, lg, c.opcode[j0 + j - 1], true, dt, t)) ok = false;
    }
  }
  // team sums of the per-thread partials
  for (int q = 0; q < npar; ++q) {
    const double sum = tsum(t, acc[q]) * trsg;  // d log|Tr| = dTr / Tr, Tr = trsg exp(trlg)
    if (t.tid == 0) gpar[(size_t)chain * npar + q] = ok ? sum : 0.0;
  }
  if (t.tid == 0) logw[2 * (size_t)chain + 1] = ok ? trlg - g.beta * m.egs : -DHUGE;
  // the checkpoints extended here stay valid for the configuration
  if (warp == 0) store_hdr(gh, c.h, lane);
}

// Largest operator count of a time bin over the chains of a group.
__global__ void k_max_bin(const __grid_constant__ DGroup g, int* out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= g.nchains) return;
  const int* bs = (const int*)(g.base + (size_t)c * g.stride + g.o_bstart);
  int mx = 0;
  for (int b = 0; b < (1 << g.L); ++b) mx = max(mx, bs[b + 1] - bs[b]);
  atomicMax(out, mx);
}

// set_mc_config: operator arrays from a time-ordered list already written
// into optau/opcode by the host (K in the header); rebuilds the sorted
// arrays, the tree, the trace, and the inverse hybridisation matrices by
// Gauss-Jordan elimination with partial pivoting (get_InvFullHybr,
// Trace.F90:2279-2336), in rank order (slot = rank).
__device__ void rebuild_minv(Ctx& c, double* maxdev, bool replace, double& dlog, double& dsign) {
  Hdr& h = *c.h;
  const DModel& m = *c.m;
  dlog = 0.0;
  dsign = 1.0;
  double* A = c.dense;  // needs kcap*kcap*2 doubles of scratch
  for (int f = 0; f < m.nf; ++f) {
    int k = h.k[f];
    if (k == 0) continue;
    const int ld = c.kcap;
    const double* I = A + (size_t)ld * ld;
    if (!gj_inverse(c, f, k, srt_ptr(c, f, 0), srt_ptr(c, f, 1), A, dlog, dsign)) {
      dlog = -DHUGE;
      dsign = 0.0;
      continue;
    }
    // I = H^{-1}: rows are c ranks, columns a ranks.  Compare / install in
    // slot order: M[slot_a][slot_c] = Inv(rank_c, rank_a)
    const short* slc = sslot_ptr(c, f, 0);
    const short* sla = sslot_ptr(c, f, 1);
    double* Mf = M_ptr(c, f);
    double dev = 0.0;
    for (int e = c.lane; e < k * k; e += 32) {
      int rc = e % k, ra = e / k;
      double val = I[(size_t)ra * ld + rc];
      size_t idx = (size_t)sla[ra] * ld + slc[rc];
      dev = fmax(dev, fabs(Mf[idx] - val));
      if (replace) Mf[idx] = val;
    }
    dev = wmax(dev);
    if (maxdev && c.lane == 0) *maxdev = fmax(*maxdev, dev);
    __syncwarp();
  }
}

// The periodic rebuild (see refresh_due): per-flavour inverse matrices, or
// the full matrix in block order for off-diagonal groups.
__device__ NOINL void ph_refresh(Ctx& c) {
  Hdr& h = *c.h;
  double dlog = 0.0, dsign = 1.0;
  if (c.g->offdiag) {
    const int K = h.K, k = K / 2, ld = c.kcap;
    if (k > 0) {
      if (od_full_inverse(c, K, dlog, dsign)) {
        const double* I = c.dense + (size_t)ld * ld;
        double* Mw = M_ptr(c, 0);
        double dev = 0.0;
        for (int e = c.lane; e < k * k; e += 32) {
          const size_t idx = (size_t)(e / k) * ld + (e % k);
          dev = fmax(dev, fabs(Mw[idx] - I[idx]));
          Mw[idx] = I[idx];
        }
        dev = wmax(dev);
        if (c.lane == 0) h.drift_m = fmax(h.drift_m, dev);
      } else {
        dlog = -DHUGE;
        dsign = 0.0;
      }
    }
  } else {
    rebuild_minv(c, &h.drift_m, true, dlog, dsign);
  }
  if (c.lane == 0) {
    h.acc_since_refresh = 0;
    h.n_refresh++;
    if (dsign != 0.0) {  // a singular rebuild keeps the fast-updated weights
      h.drift_det = fmax(h.drift_det, fabs(dlog - h.det_log));
      if (dsign != h.det_sign) h.refresh_sign_err++;
      h.det_log = dlog;
      h.det_sign = dsign;
    }
  }
  __syncwarp();
}

// set_mc_config for chains chain0 .. chain0 + nset - 1 of a group, one warp
// per chain: chain chain0 + w takes the time-ordered operators
// offs[w] .. offs[w + 1] (codes 2f + ca) and outer superstate outers[w] from
// the staging arrays, then rebuilds the per-flavour lists, the tree, the
// trace, the inverse hybridisation matrices and the sign.
__global__ void __launch_bounds__(WPB * 32) k_set_configs(const __grid_constant__ DModel m, const __grid_constant__ DGroup g,
                                                         int chain0, int nset, const int* __restrict__ offs,
                                                         const double* __restrict__ taus,
                                                         const int* __restrict__ codes,
                                                         const int* __restrict__ outers) {
  __shared__ Hdr hs[WPB];
  const int warp = threadIdx.x >> 5;
  const int w = blockIdx.x * WPB + warp;
  if (w >= nset) return;
  const int chain = chain0 + w;
  Ctx c = make_ctx(&m, &g, &hs[warp], chain);
  Hdr* gh = (Hdr*)(g.base + (size_t)chain * g.stride + g.o_hdr);
  load_hdr(c.h, gh, c.lane);
  Hdr& h = *c.h;
  const int o0 = offs[w], K = offs[w + 1] - o0, outer_sst = outers[w];
  for (int i = c.lane; i < K; i += 32) {
    c.optau[i] = taus[o0 + i];
    c.opcode[i] = codes[o0 + i];
  }
  if (c.lane == 0) h.K = K;
  __syncwarp();
  // per-flavour sorted arrays, slot = rank
  for (int f = 0; f < m.nf; ++f) {
    for (int ca = 0; ca < 2; ++ca) {
      double* st = srt_ptr(c, f, ca);
      short* ss = sslot_ptr(c, f, ca);
      double* tt = stau_ptr(c, f, ca);
      int n = 0;
      for (int base = 0; base < K; base += 32) {
        int i = base + c.lane;
        bool is = i < K && c.opcode[i] == 2 * f + ca;
        unsigned bal = __ballot_sync(FULL, is);
        int pos = n + __popc(bal & ((1u << c.lane) - 1u));
        if (is && pos < c.kcap) {
          st[pos] = c.optau[i];
          ss[pos] = (short)pos;
          tt[pos] = c.optau[i];
        }
        n += __popc(bal);
      }
      if (ca == 0 && c.lane == 0) h.k[f] = n;
    }
  }
  __syncwarp();
  if (c.lane == 0) h.outer_sst = outer_sst;
  __syncwarp();
  tree_build_all(c);
  chk_invalidate(c);
  double lg, sg;
  if (c.mono) {
    double mx, sum;
    root_trace(c, 0, h.outer_sst, mx, sum);
    trace_log(mx, sum, lg, sg);
  } else {
    Mod md;
    md.type = 0;
    dense_trace(c, md, h.outer_sst, lg, sg, solo_team(c));
  }
  double dlog, dsign;
  rebuild_minv(c, nullptr, true, dlog, dsign);
  if (c.lane == 0) {
    h.trace_log = lg;
    h.trace_sign = sg;
    h.det_log = dlog;
    h.det_sign = dsign;
    h.npairs = -1;
  }
  __syncwarp();
  double sgn = config_sign(c);
  if (c.lane == 0) h.cfgsign = -sgn;
  store_hdr(gh, c.h, c.lane);
}

// get_mc_config for chains chain0 .. chain0 + n - 1 of a group, one warp per
// chain: with offs == nullptr the operator counts and outer superstates,
// else the time-ordered operators of chain chain0 + w into
// taus/codes[offs[w] ..].
__global__ void __launch_bounds__(WPB * 32) k_get_configs(const __grid_constant__ DGroup g, int chain0, int n,
                                                         const int* __restrict__ offs, int* __restrict__ counts,
                                                         int* __restrict__ outers, double* __restrict__ taus,
                                                         int* __restrict__ codes) {
  const int w = blockIdx.x * WPB + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (w >= n) return;
  const char* base = g.base + (size_t)(chain0 + w) * g.stride;
  const Hdr* gh = (const Hdr*)(base + g.o_hdr);
  const int K = gh->K;
  if (!offs) {
    if (lane == 0) {
      counts[w] = K;
      outers[w] = gh->outer_sst;
    }
    return;
  }
  const double* ot = (const double*)(base + g.o_optau);
  const int* oc = (const int*)(base + g.o_opcode);
  const int o0 = offs[w];
  for (int i = lane; i < K; i += 32) {
    taus[o0 + i] = ot[i];
    codes[o0 + i] = oc[i];
  }
}

__global__ void __launch_bounds__(WPB * 32) k_refresh(const __grid_constant__ DModel m, const __grid_constant__ DGroup g,
                                                     int replace, double* maxdev) {
  __shared__ Hdr hs[WPB];
  int warp = threadIdx.x >> 5;
  int chain = blockIdx.x * WPB + warp;
  if (chain >= g.nchains) return;
  Ctx c = make_ctx(&m, &g, &hs[warp], chain);
  Hdr* gh = (Hdr*)(g.base + (size_t)chain * g.stride + g.o_hdr);
  load_hdr(c.h, gh, c.lane);
  double dlog, dsign;
  __shared__ double dev[WPB];
  if (c.lane == 0) dev[warp] = 0.0;
  __syncwarp();
  rebuild_minv(c, &dev[warp], replace != 0, dlog, dsign);
  if (c.lane == 0) {
    unsigned long long* p = (unsigned long long*)maxdev;
    unsigned long long v = __double_as_longlong(dev[warp]);
    atomicMax(p, v);  // non-negative doubles order like their bit patterns
  }
}

// Drift statistics of every chain of a group into out (max |dM|, max
// |d log det| as bit patterns, refreshes, sign errors); reset clears them.
__global__ void k_drift(const __grid_constant__ DGroup g, unsigned long long* out, int reset) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= g.nchains) return;
  Hdr* h = (Hdr*)(g.base + (size_t)c * g.stride + g.o_hdr);
  atomicMax(&out[0], (unsigned long long)__double_as_longlong(h->drift_m));  // non-negative
  atomicMax(&out[1], (unsigned long long)__double_as_longlong(h->drift_det));
  atomicAdd(&out[2], (unsigned long long)h->n_refresh);
  atomicAdd(&out[3], (unsigned long long)h->refresh_sign_err);
  if (reset) {
    h->drift_m = 0.0;
    h->drift_det = 0.0;
    h->n_refresh = 0;
    h->refresh_sign_err = 0;
  }
}

// Clear the measurement accumulators of every chain of a group (block c =
// chain c): the region from G(tau) to the dense work space (G, G_full,
// histogram, density matrix, Legendre, outer histograms, score sums) and
// the header's measurement count and sign sum (init_counters' measurement
// part, CTQMC.F90:847-899).
__global__ void k_reset_meas(const __grid_constant__ DGroup g) {
  char* base = g.base + (size_t)blockIdx.x * g.stride;
  unsigned long long* p = (unsigned long long*)(base + g.o_gtau);
  const size_t n = (g.o_dense - g.o_gtau) / 8;  // both offsets 256-byte aligned
  for (size_t i = threadIdx.x; i < n; i += blockDim.x) p[i] = 0ull;
  if (threadIdx.x == 0) {
    Hdr* h = (Hdr*)(base + g.o_hdr);
    h->cnt_meas = 0;
    h->meas_sign = 0.0;
  }
}

// log|det H| and the absolute log|trace| (the stored trace is relative to
// exp(-beta Egs)) of every chain of a group from the chain headers.
__global__ void k_log_weights(const __grid_constant__ DModel m, const __grid_constant__ DGroup g, double* out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= g.nchains) return;
  const Hdr* h = (const Hdr*)(g.base + (size_t)c * g.stride + g.o_hdr);
  out[2 * (size_t)(g.chain0 + c)] = h->det_log;
  out[2 * (size_t)(g.chain0 + c) + 1] = h->trace_log - g.beta * m.egs;
}

// Per-chain summary of a group: operators, measurements, sign sum, proposals.
__global__ void k_chain_stats(const __grid_constant__ DGroup g, double* out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= g.nchains) return;
  const Hdr* h = (const Hdr*)(g.base + (size_t)c * g.stride + g.o_hdr);
  out[4 * (size_t)c + 0] = (double)h->K;
  out[4 * (size_t)c + 1] = (double)h->cnt_meas;
  out[4 * (size_t)c + 2] = h->meas_sign;
  out[4 * (size_t)c + 3] = (double)h->nprop;
}

// Sum of the G(tau) accumulators, signs and measurement counts over the
// chains of a group (one thread per bin, chains strided).
__global__ void k_group_sum(const __grid_constant__ DGroup g, int nbins, double* out, double* sign_out,
                            long long* cnt_out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nbins) {
    double acc = 0.0;
    for (int c = 0; c < g.nchains; ++c) acc += ((const double*)(g.base + (size_t)c * g.stride + g.o_gtau))[i];
    out[i] = acc;
  }
  if (i == 0) {
    double ss = 0.0;
    long long cn = 0;
    for (int c = 0; c < g.nchains; ++c) {
      const Hdr* h = (const Hdr*)(g.base + (size_t)c * g.stride + g.o_hdr);
      ss += h->meas_sign;
      cn += h->cnt_meas;
    }
    *sign_out = ss;
    *cnt_out = cn;
  }
}

__global__ void k_set_window(const __grid_constant__ DModel m, const __grid_constant__ DGroup g, double tdm) {
  __shared__ Hdr hs[WPB];
  int warp = threadIdx.x >> 5;
  int chain = blockIdx.x * WPB + warp;
  if (chain >= g.nchains) return;
  Ctx c = make_ctx(&m, &g, &hs[warp], chain);
  Hdr* gh = (Hdr*)(g.base + (size_t)chain * g.stride + g.o_hdr);
  load_hdr(c.h, gh, c.lane);
  init_window(c, tdm);
  store_hdr(gh, c.h, c.lane);
}

// ---------------------------------------------------------------------------
// Host side
namespace {
thread_local std::string g_err;
int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}
#define CK(x)                                                                                     \
  do {                                                                                            \
    cudaError_t e_ = (x);                                                                         \
    if (e_ != cudaSuccess) return fail(CTHYB_ERR_CUDA, std::string(#x ": ") + cudaGetErrorString(e_)); \
  } while (0)

template <class T>
T* dev_upload(const std::vector<T>& v, cudaError_t& err) {
  T* p = nullptr;
  size_t n = std::max<size_t>(v.size(), 1) * sizeof(T);
  err = cudaMalloc(&p, n);
  if (err != cudaSuccess) return nullptr;
  if (!v.empty()) err = cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
  return p;
}
size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }
}  // namespace

}  // namespace cthyb

using namespace cthyb;

struct cthyb_model_s {
  HostModel hm;
  DModel dm;
  std::vector<void*> allocs;
  bool uploaded = false;
  int ndir = 0;                 // Hamiltonian directions set by cthyb_model_set_directions
  double* d_dir = nullptr;      // their eigenbasis blocks on the device (ndir x dm_size)
};

struct GroupHost {
  cthyb_group_desc desc;
  DGroup g;
  std::vector<double> hybr;
  double* d_hybr = nullptr;
  double* d_hybr_full = nullptr;
  double* d_empty = nullptr;
  double* d_score = nullptr;
  double* d_edges = nullptr;
  long long* d_ekeys = nullptr;
  int* d_sym = nullptr;
  int* d_seeds = nullptr;
  double* d_tdm = nullptr;
  int chain0 = 0;
};

struct cthyb_batch_s {
  cthyb_model_t model;
  std::vector<GroupHost> groups;
  char* slab = nullptr;
  int* d_err = nullptr;
  double* d_dev = nullptr;
  cudaStream_t stream = nullptr;
  int nchains = 0;
  int use_graphs = 0;
  int sync_warps = -1;  // -1: automatic; 0: independent warps (k_sweep); n: phase-synchronous blocks of n warps
  size_t sync_smem = 48 * 1024;  // dynamic shared memory the sync kernel is opted in for
  int smem_sm = 0, smem_rsv = 0; // shared memory per multiprocessor and reserved per block (bytes)
  int smem_optin = 0;           // opt-in shared memory per block (bytes)
  // captured launch sequences of warmup(n) / measure(n), replayed while n and
  // the schedule stay the same
  struct Graph {
    long long n = -1;
    int sched = -2;
    cudaGraphExec_t exec = nullptr;
  } gwarm, gmeas;
  int team = 0;         // > 0: team sweep with `team` warps per chain (k_sweep_team)
  int team_bps = 0;     // resident team blocks per multiprocessor (0: as many as fit)
  int* d_order = nullptr;   // chain order of the team sweep
  int* d_counter = nullptr; // its fetch counter
  int team_attr = 0;        // shared memory the team kernels are opted in for
  int nsm = 0;          // multiprocessors of the device
  long long logcap = 0;
  bool counters_reset_pending = false;
  double* d_red = nullptr;
  std::vector<double> red_host;
  DGroup* d_groups = nullptr;
};

static int upload_groups(cthyb_batch_s* B) {
  std::vector<DGroup> gs;
  for (GroupHost& G : B->groups) gs.push_back(G.g);
  if (!B->d_groups) CK(cudaMalloc(&B->d_groups, sizeof(DGroup) * gs.size()));
  CK(cudaMemcpy(B->d_groups, gs.data(), sizeof(DGroup) * gs.size(), cudaMemcpyHostToDevice));
  return CTHYB_OK;
}

extern "C" {

const char* cthyb_last_error(void) { return g_err.c_str(); }

int cthyb_model_create(int nd, const double* umatrix, const double* muimp, const char* qns,
                       cthyb_model_t* out) {
  if (!umatrix || !muimp || !out) return fail(CTHYB_ERR_ARG, "null argument");
  cthyb_model_s* M = new cthyb_model_s;
  std::string err;
  if (!build_model(nd, umatrix, muimp, qns, M->hm, err)) {
    delete M;
    return fail(CTHYB_ERR_ARG, err);
  }
  if (M->hm.nf > NFMAX) {
    delete M;
    return fail(CTHYB_ERR_UNSUPPORTED, "too many flavours");
  }
  *out = M;
  return CTHYB_OK;
}

// Device copy of the model tables, made on first use by a batch.
static int model_upload(cthyb_model_t M) {
  if (M->uploaded) return CTHYB_OK;
  HostModel& hm = M->hm;
  DModel& d = M->dm;
  d.nd = hm.nd;
  d.nf = hm.nf;
  d.ns = hm.ns;
  d.nss = hm.nss;
  d.nsmax = hm.nsmax;
  d.monomial = hm.monomial;
  d.mono_lv0 = 1;
  for (double x : hm.mono_lv)
    if (x != 0.0) d.mono_lv0 = 0;
  d.egs = hm.egs;
  cudaError_t e = cudaSuccess;
  auto up = [&](auto& vec) {
    auto* p = dev_upload(vec, e);
    M->allocs.push_back((void*)p);
    return p;
  };
  d.sst_n = up(hm.sst_n);
  d.sst_off = up(hm.sst_off);
  d.connect = up(hm.connect);
  d.eval = up(hm.eval);
  {
    std::vector<double> evs(hm.ns);
    for (int i = 0; i < hm.ns; ++i) evs[i] = hm.eval[i] - hm.egs;
    d.evs = up(evs);
  }
  d.has_szt = hm.has_szt;
  {
    // superstate of the spin-flipped first basis state of each superstate
    std::vector<int> sst_of_fock((size_t)1 << hm.nf, -1), sflip(hm.nss, 0);
    for (int s = 0; s < hm.nss; ++s)
      for (int i = 0; i < hm.sst_n[s]; ++i) sst_of_fock[hm.occ_fock[hm.sst_off[s] + i]] = s;
    for (int s = 0; s < hm.nss; ++s) {
      const int st = hm.occ_fock[hm.sst_off[s]];
      const int down = st & ((1 << hm.nd) - 1), upb = (st >> hm.nd) & ((1 << hm.nd) - 1);
      const int t = sst_of_fock[upb | (down << hm.nd)];
      sflip[s] = t >= 0 ? t : s;
    }
    d.sflip_sst = up(sflip);
  }
  d.mono_tgt = up(hm.mono_tgt);
  d.mono_lv = up(hm.mono_lv);
  d.mono_neg = up(hm.mono_neg);
  d.blk_off = up(hm.blk_off);
  d.blk = up(hm.blk);
  d.dm_off = up(hm.dm_off);
  d.dm_size = hm.dm_size;
  if (e != cudaSuccess) {
    for (void* p : M->allocs) cudaFree(p);
    M->allocs.clear();
    return fail(CTHYB_ERR_CUDA, std::string("model upload: ") + cudaGetErrorString(e));
  }
  M->uploaded = true;
  return CTHYB_OK;
}

int cthyb_model_set_directions(cthyb_model_t m, int nparams, const double* dumatrix, const double* dmuimp) {
  if (!m || nparams < 0 || nparams > NPARMAX || (nparams > 0 && !dumatrix && !dmuimp))
    return fail(CTHYB_ERR_ARG, "bad arguments (nparams must be 0..32)");
  std::vector<double> blocks;
  direction_blocks(m->hm, nparams, dumatrix, dmuimp, blocks);
  if (m->d_dir) {
    CK(cudaFree(m->d_dir));
    m->d_dir = nullptr;
  }
  m->ndir = 0;
  if (nparams > 0) {
    CK(cudaMalloc(&m->d_dir, blocks.size() * sizeof(double)));
    CK(cudaMemcpy(m->d_dir, blocks.data(), blocks.size() * sizeof(double), cudaMemcpyHostToDevice));
    m->ndir = nparams;
  }
  return CTHYB_OK;
}

int cthyb_model_destroy(cthyb_model_t m) {
  if (!m) return CTHYB_OK;
  if (m->d_dir) cudaFree(m->d_dir);
  for (void* p : m->allocs) cudaFree(p);
  delete m;
  return CTHYB_OK;
}

int cthyb_model_info(cthyb_model_t m, int* nsst, int* nstates, int* nsmax, int* monomial, double* egs) {
  if (!m) return fail(CTHYB_ERR_ARG, "null model");
  if (nsst) *nsst = m->hm.nss;
  if (nstates) *nstates = m->hm.ns;
  if (nsmax) *nsmax = m->hm.nsmax;
  if (monomial) *monomial = m->hm.monomial;
  if (egs) *egs = m->hm.egs;
  return CTHYB_OK;
}

int cthyb_model_states(cthyb_model_t m, int* sst_size, int* sst_offset, int* fock_state, double* evals) {
  if (!m) return fail(CTHYB_ERR_ARG, "null model");
  const HostModel& h = m->hm;
  for (int s = 0; s < h.nss; ++s) {
    if (sst_size) sst_size[s] = h.sst_n[s];
    if (sst_offset) sst_offset[s] = h.sst_off[s];
  }
  for (int i = 0; i < h.ns; ++i) {
    if (fock_state) fock_state[i] = h.fock_of[i];
    if (evals) evals[i] = h.eval[i];
  }
  return CTHYB_OK;
}

int cthyb_model_basis(cthyb_model_t m, int* occ_fock, double* evec) {
  if (!m) return fail(CTHYB_ERR_ARG, "null model");
  const HostModel& h = m->hm;
  if (occ_fock)
    for (int i = 0; i < h.ns; ++i) occ_fock[i] = h.occ_fock[i];
  if (evec) {
    std::fill(evec, evec + (size_t)h.ns * h.ns, 0.0);
    for (int s = 0; s < h.nss; ++s) {
      const int n = h.sst_n[s], o = h.sst_off[s];
      const double* v = h.evec.data() + h.evec_off[s];
      for (int k = 0; k < n; ++k)
        for (int i = 0; i < n; ++i) evec[(size_t)(o + k) * h.ns + (o + i)] = v[(size_t)k * n + i];
    }
  }
  return CTHYB_OK;
}

int cthyb_model_connect(cthyb_model_t m, int sst, int b, int s, int ca) {
  if (!m) return fail(CTHYB_ERR_ARG, "null model");
  const HostModel& h = m->hm;
  if (sst < 0 || sst >= h.nss || b < 1 || b > h.nd || s < 1 || s > 2 || ca < 1 || ca > 2) return -1;
  return h.connect[((size_t)sst * h.nf + 2 * (b - 1) + (s - 1)) * 2 + (ca - 1)];
}

static int layout_group(cthyb_batch_s* B, GroupHost& G, long long logcap) {
  const HostModel& hm = B->model->hm;
  DGroup& g = G.g;
  const cthyb_group_desc& d = G.desc;
  const int nf = hm.nf;
  g.nchains = d.nchains;
  g.beta = d.beta;
  g.hscale = (double)(d.nftau - 1) / d.beta;
  g.gscale = (double)d.ntau / d.beta;
  g.nftau = d.nftau;
  g.ntau = d.ntau;
  g.ncorr = d.ncorr > 0 ? d.ncorr : 100;
  g.maxhisto = d.maxhisto > 1 ? d.maxhisto : 500;
  g.p_outer = d.p_outer;
  g.p_global = d.p_global;
  g.p_shift = d.p_shift;
  g.p_4op = d.p_4op;
  g.dense = (d.flags & CTHYB_FLAG_DENSE) ? 1 : 0;
  g.dmma = (d.flags & CTHYB_FLAG_DMMA) ? 1 : 0;
  g.refresh_every = d.refresh_every == 0 ? CTHYB_REFRESH_DEFAULT : (d.refresh_every < 0 ? 0 : d.refresh_every);
  g.meas_dm = (d.flags & CTHYB_FLAG_NO_DM) ? 0 : 1;
  int kcap = d.kcap > 0 ? d.kcap : std::max(32, (int)std::min(4096.0, 32.0 * std::ceil(d.beta * 1.0 / 32.0 + 1.0)));
  kcap = (kcap + 3) / 4 * 4;
  int opcap = d.opcap > 0 ? d.opcap : std::max(64, std::min(nf * kcap * 2, (int)(64 + 16 * d.beta)));
  g.kcap = kcap;
  g.opcap = opcap;
  // Default depth: two leaves up to 512 operators, beyond that leaves of at
  // most 128 operators of capacity (measured optimum of the phase-
  // synchronous sweep for density-density models: at beta = 100 with
  // opcap 1024 depth 3 beats depth 2 by 2 % of the batch rate, at beta = 50
  // with opcap 512 depth 1 beats depth 2; the leaf rebuild grows with the
  // operators of a bin, the combine steps with the depth).
  int L = d.tree_levels;
  if (L < 0) {
    L = 0;  // one leaf: every proposal rewalks all operators, no combine steps
  } else if (L == 0) {
    L = 1;
    if (opcap > 512)
      while ((128ll << L) < opcap && L < 10) ++L;
  }
  if (L > 10) L = 10;  // the sweep keeps 2^(L+1) active bits per chain in shared memory
  g.L = L;
  g.binscale = (double)(1 << L) / d.beta;
  const bool mono = hm.monomial && !g.dense;
  size_t nb = mono ? (size_t)hm.ns * 10 : 0;
  nb += (size_t)hm.nss * 2;
  g.node_bytes = align_up(nb, 16);
  size_t nodes = (size_t)2 << L;  // heap indices 0 .. 2^(L+1)-1
  size_t off = 0;
  g.o_hdr = off;
  off = align_up(off + sizeof(Hdr), 256);
  g.o_mt = off;
  off = align_up(off + 624 * 4, 256);
  g.o_optau = off;
  off = align_up(off + (size_t)(opcap + 2) * 8, 256);
  g.o_opcode = off;
  off = align_up(off + (size_t)(opcap + 2) * 4, 256);
  g.o_srt_tau = off;
  off = align_up(off + (size_t)nf * 2 * kcap * 8, 256);
  g.o_srt_slot = off;
  off = align_up(off + (size_t)nf * 2 * kcap * 2, 256);
  g.o_slot_tau = off;
  off = align_up(off + (size_t)nf * 2 * kcap * 8, 256);
  g.o_M = off;
  off = align_up(off + (size_t)nf * kcap * kcap * 8, 256);
  g.o_tree = off;
  off = align_up(off + nodes * 2 * g.node_bytes, 256);
  g.o_act = off;
  off = align_up(off + nodes, 256);
  g.o_bstart = off;
  off = align_up(off + ((size_t)(1 << L) + 1) * 4, 256);
  g.o_scr = off;
  off = align_up(off + (size_t)(4 * kcap + 2 * (opcap + 2) + 2 * (opcap + 3)) * 8 + (size_t)2 * (opcap + 2) * 4, 256);
  g.o_gtau = off;
  off = align_up(off + (size_t)nf * d.ntau * 8, 256);
  g.offdiag = d.ftau_full ? 1 : 0;
  g.o_gfull = 0;
  if (g.offdiag) {
    g.o_gfull = off;
    off = align_up(off + (size_t)nf * nf * d.ntau * 8, 256);
  }
  g.o_histo = off;
  off = align_up(off + (size_t)nf * g.maxhisto * 8, 256);
  g.o_dm = off;  // diagonal (monomial models) or the superstate blocks of rho
  off = align_up(off + (size_t)(mono ? hm.ns : hm.dm_size) * 8, 256);
  g.nleg = d.nleg > 0 ? d.nleg : 0;
  g.o_gleg = off;  // GLeg (nf x nleg), or GLeg_full (nf x nf x nleg) for off-diagonal groups
  off = align_up(off + (size_t)nf * (d.ftau_full ? nf : 1) * g.nleg * 8, 256);
  g.o_outer = off;  // outer superstate/state histograms, signs, trace contributions
  off = align_up(off + (size_t)3 * (hm.nss + hm.ns) * 8, 256);
  g.nscore = (d.nscore > 0 && d.score_dE && mono) ? std::min(d.nscore, 32) : 0;
  g.o_score = off;
  off = align_up(off + (size_t)g.nscore * (1 + (size_t)nf * d.ntau) * 8, 256);
  g.o_accpair = 0;
  if (d.flags & CTHYB_FLAG_ACCPAIR) {
    g.o_accpair = off;
    off = align_up(off + (size_t)nf * d.ntau * 8, 256);
  }
  g.o_dense = off;
  size_t dense = std::max((size_t)2 * hm.nsmax * hm.nsmax + 2 * hm.nsmax, (size_t)2 * kcap * kcap) * 8;
  off = align_up(off + dense, 256);
  g.o_log = off;
  g.logcap = logcap;
  off = align_up(off + (size_t)logcap * sizeof(cthyb_record), 256);
  g.o_chk = 0;
  g.chk_bytes = 0;
  if (!mono) {
    g.chk_bytes = align_up(16 + (size_t)8 * hm.nsmax + (size_t)8 * hm.nsmax * hm.nsmax, 16);
    g.o_chk = off;
    off = align_up(off + (size_t)2 * ((1u << L) + 1) * g.chk_bytes, 256);
  }
  g.o_glscr = 0;
  if (g.nleg > 0) {
    g.o_glscr = off;
    off = align_up(off + (size_t)32 * g.nleg * 8, 256);
  }
  // work space of global, tau-shift and 4-operator moves: new inverse
  // matrices, new sorted lists, copy of the operator arrays
  g.o_glob = 0;
  if (d.p_global > 0.0 || d.p_shift > 0.0 || d.p_4op > 0.0 || d.ftau_full) {
    g.o_glob = off;
    off = align_up(off + ((size_t)nf * kcap * kcap + (size_t)nf * 2 * kcap + (opcap + 2)) * 8 +
                             (size_t)(opcap + 2) * 4,
                   256);
  }
  g.stride = off;
  return CTHYB_OK;
}

// Chain slabs come from the device's stream-ordered memory pool, which is
// told to keep freed memory for the process (release threshold at its
// maximum): a driver that creates a batch per solve (one per DMFT
// iteration) reuses the previous slab instead of mapping gigabytes anew.
static cudaError_t slab_alloc(char** p, size_t n, cudaStream_t s) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  cudaMemPool_t pool;
  if (e == cudaSuccess) e = cudaDeviceGetDefaultMemPool(&pool, dev);
  if (e == cudaSuccess) {
    uint64_t keep = ~0ull;
    e = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  if (e == cudaSuccess) e = cudaMallocAsync((void**)p, n, s);
  return e;
}
static void slab_free(char* p, cudaStream_t s) {
  if (!p) return;
  cudaFreeAsync(p, s);
  cudaStreamSynchronize(s);
}

int cthyb_batch_create(cthyb_model_t model, int ngroups, const cthyb_group_desc* groups, cthyb_batch_t* out) {
  if (!model || ngroups < 1 || !groups || !out) return fail(CTHYB_ERR_ARG, "bad arguments");
  {
    int rc = model_upload(model);
    if (rc) return rc;
  }
  cthyb_batch_s* B = new cthyb_batch_s;
  B->model = model;
  const HostModel& hm = model->hm;
  B->groups.resize(ngroups);
  size_t total = 0;
  for (int i = 0; i < ngroups; ++i) {
    GroupHost& G = B->groups[i];
    G.desc = groups[i];
    if (G.desc.nchains < 1 || G.desc.nftau < 2 || G.desc.ntau < 1 || !(G.desc.beta > 0) || !G.desc.ftau) {
      delete B;
      return fail(CTHYB_ERR_ARG, "bad group description");
    }
    if (G.desc.ftau_full && G.desc.nscore > 0 && G.desc.score_dE) {
      delete B;
      return fail(CTHYB_ERR_UNSUPPORTED, "off-diagonal hybridisation: no score measurements");
    }
    layout_group(B, G, 0);
    G.chain0 = B->nchains;
    G.g.chain0 = G.chain0;
    B->nchains += G.desc.nchains;
    total += (size_t)G.desc.nchains * G.g.stride;
  }
  cudaError_t e = cudaStreamCreateWithFlags(&B->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = slab_alloc(&B->slab, total, B->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(B->slab, 0, total, B->stream);
  if (e == cudaSuccess) e = cudaMalloc(&B->d_err, sizeof(int));
  if (e == cudaSuccess) e = cudaMemsetAsync(B->d_err, 0, sizeof(int), B->stream);
  if (e == cudaSuccess) e = cudaMalloc(&B->d_dev, sizeof(double));
  if (e == cudaSuccess) {
    int dev = 0;
    e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&B->nsm, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&B->smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&B->smem_rsv, cudaDevAttrReservedSharedMemoryPerBlock, dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&B->smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  }
  if (e != cudaSuccess) {
    cthyb_batch_destroy(B);
    return fail(CTHYB_ERR_CUDA, std::string("batch allocation: ") + cudaGetErrorString(e));
  }
  size_t off = 0;
  for (int i = 0; i < ngroups; ++i) {
    GroupHost& G = B->groups[i];
    const cthyb_group_desc& d = G.desc;
    G.g.base = B->slab + off;
    off += (size_t)d.nchains * G.g.stride;
    G.g.err_flag = B->d_err;
    // F(tau) re-laid out per flavour f = 2b+s
    G.hybr.resize((size_t)hm.nf * d.nftau);
    for (int b = 0; b < hm.nd; ++b)
      for (int s = 0; s < 2; ++s)
        for (int t = 0; t < d.nftau; ++t)
          G.hybr[(size_t)(2 * b + s) * d.nftau + t] = d.ftau[b + hm.nd * (s + 2 * (size_t)t)];
    G.d_hybr = dev_upload(G.hybr, e);
    G.g.hybr = G.d_hybr;
    G.g.hybr_full = nullptr;
    if (d.ftau_full) {  // [f1][f2][t] with f = 2b + s
      std::vector<double> hf((size_t)hm.nf * hm.nf * d.nftau);
      for (int b1 = 0; b1 < hm.nd; ++b1)
        for (int s1 = 0; s1 < 2; ++s1)
          for (int b2 = 0; b2 < hm.nd; ++b2)
            for (int s2 = 0; s2 < 2; ++s2)
              for (int t = 0; t < d.nftau; ++t)
                hf[((size_t)(2 * b1 + s1) * hm.nf + (2 * b2 + s2)) * d.nftau + t] =
                    d.ftau_full[b1 + hm.nd * (s1 + 2 * (b2 + hm.nd * (s2 + 2 * (size_t)t)))];
      G.d_hybr_full = dev_upload(hf, e);
      G.g.hybr_full = G.d_hybr_full;
    }
    std::vector<double> w;
    empty_trace_weights(hm, d.beta, w);
    G.d_empty = dev_upload(w, e);
    G.g.empty_w = G.d_empty;
    {
      const int nbins = 1 << G.g.L;
      std::vector<double> edges(nbins + 1);
      std::vector<long long> keys(nbins + 1);
      for (int j = 0; j <= nbins; ++j) {
        edges[j] = d.beta * std::ldexp((double)j, -G.g.L);  // exact scaling, one rounding
        std::memcpy(&keys[j], &edges[j], 8);
      }
      G.d_edges = dev_upload(edges, e);
      G.d_ekeys = dev_upload(keys, e);
      G.g.edges = G.d_edges;
      G.g.ekeys = G.d_ekeys;
    }
    G.g.nsym = 0;
    G.g.symmoves = nullptr;
    if (d.nsym > 0 && d.symmoves) {
      // the moves and their inverses, SymMoves(NSymMove + i, SymMoves(i, j)) = j
      const int n2 = hm.nf;
      std::vector<int> sm((size_t)2 * d.nsym * n2);
      for (int i = 0; i < d.nsym; ++i)
        for (int j = 0; j < n2; ++j) {
          const int t = d.symmoves[(size_t)i * n2 + j];
          sm[(size_t)i * n2 + j] = t;
          if (t >= 1 && t <= n2) sm[(size_t)(d.nsym + i) * n2 + (t - 1)] = j + 1;
        }
      G.d_sym = dev_upload(sm, e);
      G.g.symmoves = G.d_sym;
      G.g.nsym = d.nsym;
    }
    G.g.score_dE = nullptr;
    if (G.g.nscore > 0) {
      std::vector<double> dE(d.score_dE, d.score_dE + (size_t)G.g.nscore * hm.ns);
      G.d_score = dev_upload(dE, e);
      G.g.score_dE = G.d_score;
    }
    std::vector<int> seeds(d.nchains);
    for (int c = 0; c < d.nchains; ++c) seeds[c] = d.seeds ? d.seeds[c] : d.seed0 + c;
    G.d_seeds = dev_upload(seeds, e);
    std::vector<double> tdm(1, d.taudiff_max);
    G.d_tdm = dev_upload(tdm, e);
    if (e != cudaSuccess) {
      cthyb_batch_destroy(B);
      return fail(CTHYB_ERR_CUDA, std::string("group upload: ") + cudaGetErrorString(e));
    }
    int nblk = (d.nchains + WPB - 1) / WPB;
    k_init<<<nblk, WPB * 32, 0, B->stream>>>(model->dm, G.g, G.d_seeds, G.d_tdm, G.g.ncorr);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
      cthyb_batch_destroy(B);
      return fail(CTHYB_ERR_CUDA, std::string("init launch: ") + cudaGetErrorString(e));
    }
  }
  e = cudaStreamSynchronize(B->stream);
  if (e != cudaSuccess) {
    cthyb_batch_destroy(B);
    return fail(CTHYB_ERR_CUDA, std::string("init: ") + cudaGetErrorString(e));
  }
  if (int rc = upload_groups(B)) {
    cthyb_batch_destroy(B);
    return rc;
  }
  *out = B;
  return CTHYB_OK;
}

int cthyb_batch_destroy(cthyb_batch_t B) {
  if (!B) return CTHYB_OK;
  if (B->stream) cudaStreamSynchronize(B->stream);
  for (GroupHost& G : B->groups) {
    cudaFree(G.d_hybr);
    cudaFree(G.d_hybr_full);
    cudaFree(G.d_empty);
    cudaFree(G.d_score);
    cudaFree(G.d_edges);
    cudaFree(G.d_ekeys);
    cudaFree(G.d_sym);
    cudaFree(G.d_seeds);
    cudaFree(G.d_tdm);
  }
  if (B->stream) slab_free(B->slab, B->stream);
  cudaFree(B->d_err);
  cudaFree(B->d_dev);
  if (B->d_red) cudaFree(B->d_red);
  if (B->d_order) cudaFree(B->d_order);
  if (B->d_counter) cudaFree(B->d_counter);
  if (B->d_groups) cudaFree(B->d_groups);
  if (B->gwarm.exec) cudaGraphExecDestroy(B->gwarm.exec);
  if (B->gmeas.exec) cudaGraphExecDestroy(B->gmeas.exec);
  if (B->stream) cudaStreamDestroy(B->stream);
  delete B;
  return CTHYB_OK;
}

int cthyb_batch_nchains(cthyb_batch_t B) { return B ? B->nchains : 0; }

int cthyb_batch_stream(cthyb_batch_t B, void** s) {
  if (!B || !s) return fail(CTHYB_ERR_ARG, "null");
  *s = (void*)B->stream;
  return CTHYB_OK;
}

int cthyb_batch_use_graphs(cthyb_batch_t B, int on) {
  if (!B) return fail(CTHYB_ERR_ARG, "null");
  B->use_graphs = on;
  return CTHYB_OK;
}

int cthyb_batch_set_taudiffmax(cthyb_batch_t B, int group, double tdm) {
  if (!B || group < 0 || group >= (int)B->groups.size()) return fail(CTHYB_ERR_ARG, "bad group");
  GroupHost& G = B->groups[group];
  int nblk = (G.desc.nchains + WPB - 1) / WPB;
  k_set_window<<<nblk, WPB * 32, 0, B->stream>>>(B->model->dm, G.g, tdm);
  CK(cudaGetLastError());
  return CTHYB_OK;
}

// Warps per block of the sweep: the set value, or the automatic choice --
// phase-synchronous blocks, two per multiprocessor, chains spread evenly
// over the multiprocessors (at 64 registers a thread an SM holds 32 chain
// warps).
static int schedule_of(cthyb_batch_t B) {
  int nw = B->sync_warps;
  if (nw < 0) nw = std::min(16, std::max(1, (B->nchains + 2 * B->nsm - 1) / (2 * std::max(B->nsm, 1))));
  return nw;
}

// One chain per block and at most one block per multiprocessor: the
// chain's operator arrays, sorted lists, tree, bin starts and scratch live
// in the block's shared memory for the launch (resident_enter).  Returns
// the bytes of that area (0: not resident) and aligns `smem`, the per-warp
// area in front of it.
static size_t sync_resident(cthyb_batch_t B, int nw, size_t& smem) {
  size_t resident = 0;
  if (nw == 1 && B->nchains <= B->nsm) {
    for (GroupHost& G : B->groups) resident = std::max(resident, resident_bytes(G.g));
    smem = align_up(smem, 16);
    if (smem + resident > (size_t)B->smem_optin) resident = 0;
  }
  return resident;
}

// Shared memory of the sync kernel: opt in for `smem` bytes a block and
// ask for the smallest carveout that holds `blocks` such blocks (two; one
// for a resident chain, whose warp's stack then keeps L1), leaving the
// rest of the multiprocessor's 256 KB to the L1 cache (the chains' hot
// arrays live there; a carveout of 10 % against the default measured +1 %,
// 50 % -3 %, 100 % -17 % on the 4096-chain batch).
static int sync_attributes(cthyb_batch_t B, size_t smem, int blocks) {
  if (smem > B->sync_smem) {
    CK(cudaFuncSetAttribute(k_sweep_sync, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    B->sync_smem = smem;
  }
  if (B->smem_sm > 0) {
    const size_t need = (size_t)blocks * (smem + (size_t)B->smem_rsv);
    const int pct = (int)std::min<size_t>(100, (100 * need + B->smem_sm - 1) / B->smem_sm + 1);
    // a function attribute: the last value set by any batch of the process
    static int carve = -1;
    if (pct != carve) {
      CK(cudaFuncSetAttribute(k_sweep_sync, cudaFuncAttributePreferredSharedMemoryCarveout, pct));
      carve = pct;
    }
  }
  return CTHYB_OK;
}

// Team sweep: order the chains by estimated cost (k_order), reset the
// fetch counter, and launch one persistent grid of `team`-warp blocks
// (as many as fit on the device, at most one per chain).
static int launch_team(cthyb_batch_t B, long long nprop, int nmeas, int reset) {
  int Lmax = 1;
  for (GroupHost& G : B->groups) Lmax = std::max(Lmax, G.g.L);
  const int threads = 32 * B->team;
  const size_t smem = sizeof(Hdr) + sizeof(cthyb_record) + sizeof(Prop) + 32 * sizeof(double) + (2 << Lmax);
  int n2 = 1;
  while (n2 < B->nchains) n2 <<= 1;
  const size_t osmem = n2 <= ORDER_MAX ? (size_t)n2 * 8 : 0;
  if (!B->d_order) {
    CK(cudaMalloc(&B->d_order, sizeof(int) * (size_t)B->nchains));
    CK(cudaMalloc(&B->d_counter, sizeof(int)));
  }
  if (!B->team_attr) {
    CK(cudaFuncSetAttribute(k_order, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(ORDER_MAX * 8)));
    CK(cudaFuncSetAttribute(k_sweep_team, cudaFuncAttributeMaxDynamicSharedMemorySize, 48 * 1024));
    B->team_attr = 1;
  }
  int per_sm = 0;
  CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sweep_team, threads, smem));
  per_sm = std::max(per_sm, 1);
  if (B->team_bps > 0) per_sm = std::min(per_sm, B->team_bps);
  const int grid = std::max(1, std::min(B->nchains, per_sm * std::max(B->nsm, 1)));
  k_order<<<1, 1024, osmem, B->stream>>>(B->model->dm, B->d_groups, (int)B->groups.size(), B->nchains, B->d_order);
  CK(cudaGetLastError());
  CK(cudaMemsetAsync(B->d_counter, 0, sizeof(int), B->stream));
  k_sweep_team<<<grid, threads, smem, B->stream>>>(B->model->dm, B->d_groups, (int)B->groups.size(), B->nchains,
                                                  nprop, nmeas, reset, B->d_order, B->d_counter);
  CK(cudaGetLastError());
  return CTHYB_OK;
}

static int launch_sweeps(cthyb_batch_t B, long long nprop, int nmeas, int reset) {
  if (B->team > 0) return launch_team(B, nprop, nmeas, reset);
  int Lmax = 1;
  for (GroupHost& G : B->groups) Lmax = std::max(Lmax, G.g.L);
  const int actbytes = 2 << Lmax;
  const int nw = schedule_of(B);
  if (nw > 0) {
    const int nblk = (B->nchains + nw - 1) / nw;
    size_t smem = (size_t)nw * (sizeof(Hdr) + sizeof(cthyb_record) + sizeof(Prop) + actbytes);
    const size_t resident = sync_resident(B, nw, smem);
    int rc = sync_attributes(B, smem + resident, resident ? 1 : 2);
    if (rc) return rc;
    k_sweep_sync<<<nblk, nw * 32, smem + resident, B->stream>>>(B->model->dm, B->d_groups, (int)B->groups.size(),
                                                                B->nchains, nprop, nmeas, reset, actbytes,
                                                                resident ? (int)smem : 0);
  } else {
    const int nblk = (B->nchains + WPB - 1) / WPB;
    k_sweep<<<nblk, WPB * 32, (size_t)WPB * actbytes, B->stream>>>(B->model->dm, B->d_groups,
                                                                   (int)B->groups.size(), B->nchains, nprop, nmeas,
                                                                   reset, actbytes);
  }
  CK(cudaGetLastError());
  return CTHYB_OK;
}

int cthyb_batch_set_schedule(cthyb_batch_t B, int warps_per_block) {
  if (!B || warps_per_block < -1 || warps_per_block > 32) return fail(CTHYB_ERR_ARG, "warps_per_block must be -1..32");
  B->sync_warps = warps_per_block;
  B->team = 0;
  return CTHYB_OK;
}

int cthyb_batch_set_team(cthyb_batch_t B, int warps_per_chain, int blocks_per_sm) {
  if (!B || warps_per_chain < 0 || warps_per_chain > TEAM_MAX_THREADS / 32 || blocks_per_sm < 0)
    return fail(CTHYB_ERR_ARG, "warps_per_chain must be 0..16, blocks_per_sm >= 0");
  B->team = warps_per_chain;
  B->team_bps = blocks_per_sm;
  return CTHYB_OK;
}

// The launches of warmup(n) (meas = false) or measure(n); chunks keep single
// launches short.
static int issue_sweeps(cthyb_batch_t B, long long n, bool meas) {
  const long long chunk = meas ? 200 : 20000;
  int reset = 1;
  for (long long done = 0; done < n; done += chunk) {
    const long long m = std::min<long long>(chunk, n - done);
    int rc = meas ? launch_sweeps(B, 0, (int)m, reset) : launch_sweeps(B, m, 0, reset);
    if (rc) return rc;
    reset = 0;
  }
  if (n == 0 && !meas) return launch_sweeps(B, 0, 0, 1);
  return CTHYB_OK;
}

// Capture the launch sequence once per (n, schedule) and replay it.
static int graph_sweeps(cthyb_batch_t B, cthyb_batch_s::Graph& G, long long n, bool meas) {
  const int sched = B->team > 0 ? 100 + B->team + 1000 * B->team_bps : schedule_of(B);
  if (!G.exec || G.n != n || G.sched != sched) {
    if (G.exec) {
      CK(cudaGraphExecDestroy(G.exec));
      G.exec = nullptr;
    }
    // kernel attributes are set outside the capture
    int Lmax = 1;
    for (GroupHost& g : B->groups) Lmax = std::max(Lmax, g.g.L);
    if (B->team > 0) {
      // attributes, order and counter buffers set up by one eager launch
      // sequence outside the capture
      if (!B->d_order || !B->team_attr) {
        int rc = launch_team(B, 0, 0, 0);
        if (rc) return rc;
      }
    } else if (sched > 0) {
      size_t smem = (size_t)sched * (sizeof(Hdr) + sizeof(cthyb_record) + sizeof(Prop) + (2 << Lmax));
      const size_t resident = sync_resident(B, sched, smem);
      int rc = sync_attributes(B, smem + resident, resident ? 1 : 2);
      if (rc) return rc;
    }
    CK(cudaStreamBeginCapture(B->stream, cudaStreamCaptureModeThreadLocal));
    int rc = issue_sweeps(B, n, meas);
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamEndCapture(B->stream, &graph);
    if (rc) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    CK(e);
    e = cudaGraphInstantiate(&G.exec, graph, 0);
    cudaGraphDestroy(graph);
    CK(e);
    G.n = n;
    G.sched = sched;
  }
  CK(cudaGraphLaunch(G.exec, B->stream));
  return CTHYB_OK;
}

int cthyb_batch_warmup(cthyb_batch_t B, int64_t n) {
  if (!B || n < 0) return fail(CTHYB_ERR_ARG, "bad arguments");
  return B->use_graphs ? graph_sweeps(B, B->gwarm, n, false) : issue_sweeps(B, n, false);
}

int cthyb_batch_measure(cthyb_batch_t B, int64_t nmeas) {
  if (!B || nmeas < 0) return fail(CTHYB_ERR_ARG, "bad arguments");
  if (nmeas == 0) return CTHYB_OK;
  return B->use_graphs ? graph_sweeps(B, B->gmeas, nmeas, true) : issue_sweeps(B, nmeas, true);
}

int cthyb_batch_autotune(cthyb_batch_t B, int64_t nprop, int* best_out) {
  if (!B || nprop < 1) return fail(CTHYB_ERR_ARG, "bad arguments");
  // candidates: phase-synchronous blocks of n chains (0: independent
  // warps) and, for dense-block models, team sweeps of T warps per chain
  // (encoded 100 + T)
  bool dense = false;
  for (GroupHost& G : B->groups) dense = dense || !(B->model->hm.monomial && !G.g.dense);
  std::vector<int> cl = {0, 4, 8, 12, 14, 16, 20, 24, 28, 32};
  // team candidates: 100 + T warps per chain + 1000 x resident blocks per
  // multiprocessor (0: as many as fit)
  if (dense) cl = {0, 1, 104, 108, 2108, 4108, 116, 1116, 2116};
  const int ncand = (int)cl.size();
  const int* cands = cl.data();
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  const int saved = B->sync_warps, saved_team = B->team, saved_bps = B->team_bps;
  int best = saved_team > 0 ? 100 + saved_team + 1000 * saved_bps : saved;
  // two passes over the candidates, the second in reverse order, half the
  // proposals each: a drift of the chains' cost during tuning (expansion
  // orders still growing) then weighs on every candidate alike
  std::vector<float> tot(ncand, 0.f);
  int rc = CTHYB_OK;
  const long long half = std::max<long long>(1, nprop / 2);
  for (int pass = 0; pass < 2 && rc == CTHYB_OK; ++pass)
    for (int q = 0; q < ncand; ++q) {
      const int ci = pass == 0 ? q : ncand - 1 - q;
      B->team = cands[ci] >= 100 ? cands[ci] % 1000 - 100 : 0;
      B->team_bps = cands[ci] >= 100 ? cands[ci] / 1000 : 0;
      B->sync_warps = cands[ci] >= 100 ? saved : cands[ci];
      cudaEventRecord(e0, B->stream);
      rc = issue_sweeps(B, half, false);
      if (rc) break;
      cudaEventRecord(e1, B->stream);
      if (cudaEventSynchronize(e1) != cudaSuccess) {
        rc = fail(CTHYB_ERR_CUDA, "autotune launch failed");
        break;
      }
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      tot[ci] += ms;
    }
  float best_ms = 3.4e38f;
  for (int q = 0; q < ncand && rc == CTHYB_OK; ++q)
    if (tot[q] < best_ms) {
      best_ms = tot[q];
      best = cands[q];
    }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) {
    B->sync_warps = saved;
    B->team = saved_team;
    B->team_bps = saved_bps;
  } else {
    B->team = best >= 100 ? best % 1000 - 100 : 0;
    B->team_bps = best >= 100 ? best / 1000 : 0;
    B->sync_warps = best >= 100 ? saved : best;
  }
  if (best_out) *best_out = B->team > 0 ? 100 + B->team + 1000 * B->team_bps : B->sync_warps;
  return rc;
}

int cthyb_batch_reset_measurements(cthyb_batch_t B) {
  if (!B) return fail(CTHYB_ERR_ARG, "null");
  for (GroupHost& G : B->groups) {
    k_reset_meas<<<G.desc.nchains, 256, 0, B->stream>>>(G.g);
    CK(cudaGetLastError());
  }
  return CTHYB_OK;
}

int cthyb_batch_sync(cthyb_batch_t B) {
  if (!B) return fail(CTHYB_ERR_ARG, "null");
  CK(cudaStreamSynchronize(B->stream));
  int flag = 0;
  CK(cudaMemcpy(&flag, B->d_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (flag == ST_CAPACITY) return fail(CTHYB_ERR_CAPACITY, "a chain reached its operator capacity (kcap/opcap)");
  if (flag == ST_NUMERIC) return fail(CTHYB_ERR_NUMERIC, "DetRat too small in removal");
  if (flag == ST_INTERNAL) return fail(CTHYB_ERR_INTERNAL, "pair bookkeeping inconsistency");
  if (flag) return fail(CTHYB_ERR_INTERNAL, "chain error");
  return CTHYB_OK;
}

static int find_chain(cthyb_batch_t B, int chain, GroupHost** G, int* local) {
  if (!B || chain < 0 || chain >= B->nchains) return fail(CTHYB_ERR_ARG, "bad chain index");
  for (GroupHost& g : B->groups)
    if (chain >= g.chain0 && chain < g.chain0 + g.desc.nchains) {
      *G = &g;
      *local = chain - g.chain0;
      return CTHYB_OK;
    }
  return fail(CTHYB_ERR_ARG, "bad chain index");
}

static int read_hdr(cthyb_batch_t B, GroupHost* G, int c, Hdr& h) {
  CK(cudaStreamSynchronize(B->stream));
  CK(cudaMemcpy(&h, G->g.base + (size_t)c * G->g.stride + G->g.o_hdr, sizeof(Hdr), cudaMemcpyDeviceToHost));
  return CTHYB_OK;
}

int cthyb_batch_state(cthyb_batch_t B, int chain, double* o) {
  GroupHost* G;
  int c;
  int rc = find_chain(B, chain, &G, &c);
  if (rc) return rc;
  Hdr h;
  rc = read_hdr(B, G, c, h);
  if (rc) return rc;
  o[0] = h.trace_log;
  o[1] = h.trace_sign;
  o[2] = h.det_log;
  o[3] = h.det_sign;
  o[4] = h.cfgsign;
  o[5] = h.npairs;
  o[6] = h.outer_sst;
  o[7] = h.window_position;
  o[8] = h.num_windows;
  o[9] = h.K;
  o[10] = h.tauwin_min;
  o[11] = h.tauwin_max;
  o[12] = h.taudiff_max;
  o[13] = h.nslide;
  o[14] = h.status;
  o[15] = h.k[0];
  return CTHYB_OK;
}

int cthyb_batch_results_extra(cthyb_batch_t B, int chain, double* gleg, double* outer_sst_histo,
                              double* outer_state_histo, double* sign_sst, double* sign_state,
                              double* contrib_sst, double* contrib_state) {
  GroupHost* G;
  int c;
  int rc = find_chain(B, chain, &G, &c);
  if (rc) return rc;
  Hdr h;
  rc = read_hdr(B, G, c, h);
  if (rc) return rc;
  const HostModel& hm = B->model->hm;
  char* base = G->g.base + (size_t)c * G->g.stride;
  const int nf = hm.nf, nleg = G->g.nleg, nss = hm.nss, ns = hm.ns;
  const double cnt = (double)h.cnt_meas;
  const double ms = h.cnt_meas ? h.meas_sign / cnt : 0.0;
  if (gleg && nleg > 0 && G->g.offdiag) {
    // MeasGtauRem_full fills GLeg_full only (CTQMC.F90:8561-8566)
    std::fill(gleg, gleg + (size_t)nf * nleg, 0.0);
  } else if (gleg && nleg > 0) {
    std::vector<double> raw((size_t)nf * nleg);
    CK(cudaMemcpy(raw.data(), base + G->g.o_gleg, raw.size() * 8, cudaMemcpyDeviceToHost));
    const double zs = h.cnt_meas ? -1.0 / (cnt * ms) : 0.0;
    for (int f = 0; f < nf; ++f)
      for (int l = 0; l < nleg; ++l) {
        // GLeg * sqrt(2l+1)/beta, then -GLeg * zScaling (CTQMC.F90:8755-8760)
        const double v = raw[(size_t)f * nleg + l] * std::sqrt(2.0 * l + 1.0) / G->g.beta;
        gleg[(f / 2) + hm.nd * ((f % 2) + 2 * (size_t)l)] = -v * zs;
      }
  }
  std::vector<double> o((size_t)3 * (nss + ns));
  CK(cudaMemcpy(o.data(), base + G->g.o_outer, o.size() * 8, cudaMemcpyDeviceToHost));
  const double* sv = o.data();
  const double* ss = sv + nss;
  const double* sc = ss + nss;
  const double* tv = sc + nss;
  const double* ts = tv + ns;
  const double* tc = ts + ns;
  // SignHisto /= visits (0/0 stays NaN as in the reference), histograms and
  // contributions / CntMeas (CTQMC.F90:8740-8752)
  for (int s = 0; s < nss; ++s) {
    if (sign_sst) sign_sst[s] = ss[s] / sv[s];
    if (outer_sst_histo) outer_sst_histo[s] = sv[s] / cnt;
    if (contrib_sst) contrib_sst[s] = sc[s] / cnt;
  }
  for (int i = 0; i < ns; ++i) {
    if (sign_state) sign_state[i] = ts[i] / tv[i];
    if (outer_state_histo) outer_state_histo[i] = tv[i] / cnt;
    if (contrib_state) contrib_state[i] = tc[i] / cnt;
  }
  return CTHYB_OK;
}

int cthyb_batch_results_score(cthyb_batch_t B, int chain, double* dgtau, double* mean_score) {
  GroupHost* G;
  int c;
  int rc = find_chain(B, chain, &G, &c);
  if (rc) return rc;
  const int ns = G->g.nscore;
  if (ns <= 0) return fail(CTHYB_ERR_ARG, "the group has no score directions");
  Hdr h;
  rc = read_hdr(B, G, c, h);
  if (rc) return rc;
  const HostModel& hm = B->model->hm;
  const int nf = hm.nf, nt = G->g.ntau;
  std::vector<double> acc((size_t)ns * (1 + (size_t)nf * nt)), gt((size_t)nf * nt);
  char* base = G->g.base + (size_t)c * G->g.stride;
  CK(cudaMemcpy(acc.data(), base + G->g.o_score, acc.size() * 8, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(gt.data(), base + G->g.o_gtau, gt.size() * 8, cudaMemcpyDeviceToHost));
  const double cnt = (double)h.cnt_meas;
  if (cnt <= 0) return fail(CTHYB_ERR_ARG, "no measurements");
  // G = -(raw/cnt)/(-mean_sign) * Ntau/beta^2 (CTQMC.F90:8730); the sign is
  // constant (+-1) in a sign-free model
  const double ms = h.meas_sign / cnt;
  const double norm = (double)nt / (G->g.beta * G->g.beta) / ms;
  for (int p = 0; p < ns; ++p) {
    const double gmean = acc[p] / cnt;
    if (mean_score) mean_score[p] = gmean;
    if (!dgtau) continue;
    for (int f = 0; f < nf; ++f)
      for (int t = 0; t < nt; ++t) {
        const double cov = acc[ns + ((size_t)p * nf + f) * nt + t] / cnt - gt[(size_t)f * nt + t] / cnt * gmean;
        dgtau[(size_t)p * nf * nt + (f / 2) + hm.nd * ((f % 2) + 2 * (size_t)t)] = cov * norm;
      }
  }
  return CTHYB_OK;
}

int cthyb_batch_results(cthyb_batch_t B, int chain, double* gtau, double* mean_sign, double* dmat,
                        double* histo, int64_t* counters) {
  GroupHost* G;
  int c;
  int rc = find_chain(B, chain, &G, &c);
  if (rc) return rc;
  Hdr h;
  rc = read_hdr(B, G, c, h);
  if (rc) return rc;
  const HostModel& hm = B->model->hm;
  char* base = G->g.base + (size_t)c * G->g.stride;
  const int nt = G->g.ntau, nf = hm.nf;
  double ms = h.cnt_meas ? h.meas_sign / (double)h.cnt_meas : 0.0;
  if (mean_sign) *mean_sign = ms;
  if (gtau) {
    std::vector<double> raw((size_t)nf * nt);
    CK(cudaMemcpy(raw.data(), base + G->g.o_gtau, raw.size() * 8, cudaMemcpyDeviceToHost));
    for (int f = 0; f < nf; ++f) {
      int b = f / 2, s = f % 2;
      for (int t = 0; t < nt; ++t) {
        double v = h.cnt_meas ? -(raw[(size_t)f * nt + t] / (double)h.cnt_meas) / (-ms) * (double)nt /
                                    (G->g.beta * G->g.beta)
                              : 0.0;
        gtau[b + hm.nd * (s + 2 * (size_t)t)] = v;
      }
    }
  }
  if (dmat) {
    const bool blocks = G->g.o_chk != 0;
    std::vector<double> d(blocks ? hm.dm_size : hm.ns);
    CK(cudaMemcpy(d.data(), base + G->g.o_dm, d.size() * 8, cudaMemcpyDeviceToHost));
    double zs = h.cnt_meas ? -1.0 / ((double)h.cnt_meas * ms) : 0.0;
    std::memset(dmat, 0, sizeof(double) * (size_t)hm.ns * hm.ns);
    if (!blocks) {
      for (int i = 0; i < hm.ns; ++i) dmat[(size_t)i * hm.ns + i] = d[i] * zs;
    } else {
      for (int sst = 0; sst < hm.nss; ++sst) {
        const int n = hm.sst_n[sst], o = hm.sst_off[sst];
        for (int s2 = 0; s2 < n; ++s2)
          for (int s1 = 0; s1 < n; ++s1)
            dmat[(size_t)(o + s2) * hm.ns + (o + s1)] = d[hm.dm_off[sst] + (size_t)s2 * n + s1] * zs;
      }
    }
  }
  if (histo) {
    const int hmx = G->g.maxhisto;
    std::vector<double> hh((size_t)nf * hmx);
    CK(cudaMemcpy(hh.data(), base + G->g.o_histo, hh.size() * 8, cudaMemcpyDeviceToHost));
    for (int f = 0; f < nf; ++f)
      for (int k = 0; k < hmx; ++k)
        histo[(f / 2) + hm.nd * ((f % 2) + 2 * (size_t)k)] =
            h.cnt_meas ? hh[(size_t)f * hmx + k] / (double)h.cnt_meas : 0.0;
  }
  if (counters) {
    counters[0] = h.try_add;
    counters[1] = h.acc_add;
    counters[2] = h.try_rem;
    counters[3] = h.acc_rem;
    counters[4] = h.qn_add;
    counters[5] = h.qn_rem;
    counters[6] = h.cnt_meas;
    counters[7] = h.nprop;
  }
  return CTHYB_OK;
}

int cthyb_batch_group_sums(cthyb_batch_t B, int group, double* gsum, double* sign_sum, int64_t* cnt) {
  if (!B || group < 0 || group >= (int)B->groups.size()) return fail(CTHYB_ERR_ARG, "bad group");
  GroupHost& G = B->groups[group];
  const HostModel& hm = B->model->hm;
  const int nt = G.g.ntau, nf = hm.nf, nbins = nf * nt;
  if ((int)B->red_host.size() < nbins + 2) {
    if (B->d_red) cudaFree(B->d_red);
  if (B->d_order) cudaFree(B->d_order);
  if (B->d_counter) cudaFree(B->d_counter);
    B->d_red = nullptr;
    CK(cudaMalloc(&B->d_red, (size_t)(nbins + 2) * 8));
    B->red_host.assign(nbins + 2, 0.0);
  }
  k_group_sum<<<(nbins + 255) / 256, 256, 0, B->stream>>>(G.g, nbins, B->d_red, B->d_red + nbins,
                                                          (long long*)(B->d_red + nbins + 1));
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(B->red_host.data(), B->d_red, (size_t)(nbins + 2) * 8, cudaMemcpyDeviceToHost, B->stream));
  CK(cudaStreamSynchronize(B->stream));
  const double* raw = B->red_host.data();
  if (gsum)
    for (int f = 0; f < nf; ++f)
      for (int t = 0; t < nt; ++t) gsum[(f / 2) + hm.nd * ((f % 2) + 2 * (size_t)t)] = raw[(size_t)f * nt + t];
  if (sign_sum) *sign_sum = raw[nbins];
  long long cn;
  std::memcpy(&cn, &raw[nbins + 1], 8);
  if (cnt) *cnt = cn;
  return CTHYB_OK;
}

int cthyb_batch_get_config(cthyb_batch_t B, int chain, int* n, double* taus, int* orbs, int* spins, int* cas,
                           int* outer) {
  GroupHost* G;
  int c;
  int rc = find_chain(B, chain, &G, &c);
  if (rc) return rc;
  Hdr h;
  rc = read_hdr(B, G, c, h);
  if (rc) return rc;
  char* base = G->g.base + (size_t)c * G->g.stride;
  std::vector<double> t(h.K);
  std::vector<int> code(h.K);
  if (h.K) {
    CK(cudaMemcpy(t.data(), base + G->g.o_optau, h.K * 8, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(code.data(), base + G->g.o_opcode, h.K * 4, cudaMemcpyDeviceToHost));
  }
  *n = h.K;
  for (int i = 0; i < h.K; ++i) {
    if (taus) taus[i] = t[i];
    int f = code[i] >> 1;
    if (orbs) orbs[i] = f / 2 + 1;
    if (spins) spins[i] = f % 2 + 1;
    if (cas) cas[i] = (code[i] & 1) + 1;
  }
  if (outer) *outer = h.outer_sst;
  return CTHYB_OK;
}

// Checks one chain's configuration (get_mc_config layout, 1-based orbital,
// spin and creator/annihilator indices) and appends it, time ordered, as
// operator codes 2f + ca to the staging arrays.
static int stage_config(cthyb_batch_t B, const GroupHost* G, int n, const double* taus, const int* orbs,
                        const int* spins, const int* cas, int outer_sst, std::vector<double>& t,
                        std::vector<int>& code) {
  const HostModel& hm = B->model->hm;
  if (n < 0 || n > G->g.opcap || outer_sst < 0 || outer_sst >= hm.nss)
    return fail(CTHYB_ERR_ARG, "configuration exceeds capacity or bad superstate");
  std::vector<int> idx(n);
  for (int i = 0; i < n; ++i) idx[i] = i;
  std::stable_sort(idx.begin(), idx.end(), [&](int a, int b) { return taus[a] < taus[b]; });
  std::vector<int> per(hm.nf * 2, 0);
  const size_t o = t.size();
  for (int i = 0; i < n; ++i) {
    int j = idx[i];
    if (orbs[j] < 1 || orbs[j] > hm.nd || spins[j] < 1 || spins[j] > 2 || cas[j] < 1 || cas[j] > 2)
      return fail(CTHYB_ERR_ARG, "bad operator");
    const double tj = taus[j];
    if (!(tj >= 0.0 && tj < G->g.beta) || (i > 0 && !(tj > t[o + i - 1])))  // in [0, beta), distinct
      return fail(CTHYB_ERR_ARG, "operator times must be distinct and in [0, beta)");
    t.push_back(tj);
    int f = 2 * (orbs[j] - 1) + (spins[j] - 1);
    code.push_back(2 * f + (cas[j] - 1));
    per[code.back()]++;
  }
  for (int f = 0; f < hm.nf; ++f) {
    if (per[2 * f] != per[2 * f + 1]) return fail(CTHYB_ERR_ARG, "unbalanced configuration");
    if (per[2 * f] > G->g.kcap) return fail(CTHYB_ERR_CAPACITY, "configuration exceeds kcap");
  }
  return CTHYB_OK;
}

// Uploads the staged configurations of chains c0 .. c0 + n - 1 of one group
// (one copy per array) and rebuilds them with k_set_configs.
static int upload_configs(cthyb_batch_t B, GroupHost* G, int c0, int n, const std::vector<int>& offs,
                          const std::vector<double>& t, const std::vector<int>& code,
                          const std::vector<int>& outer) {
  const size_t nop = t.size();
  const size_t bytes = (offs.size() + outer.size() + nop) * 4 + nop * 8 + 16;
  char* d = nullptr;
  CK(cudaMalloc(&d, bytes));
  double* dt = (double*)d;
  int* dcode = (int*)(d + nop * 8);
  int* doffs = dcode + nop;
  int* douter = doffs + offs.size();
  cudaError_t e = cudaSuccess;
  if (nop) {
    if (e == cudaSuccess) e = cudaMemcpyAsync(dt, t.data(), nop * 8, cudaMemcpyHostToDevice, B->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dcode, code.data(), nop * 4, cudaMemcpyHostToDevice, B->stream);
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(doffs, offs.data(), offs.size() * 4, cudaMemcpyHostToDevice, B->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(douter, outer.data(), outer.size() * 4, cudaMemcpyHostToDevice, B->stream);
  if (e == cudaSuccess) {
    k_set_configs<<<(n + WPB - 1) / WPB, WPB * 32, 0, B->stream>>>(B->model->dm, G->g, c0, n, doffs, dt, dcode, douter);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(B->stream);
  cudaFree(d);
  CK(e);
  return CTHYB_OK;
}

int cthyb_batch_get_configs(cthyb_batch_t B, int chain0, int nget, int* offsets, int cap, double* taus,
                            int* orbs, int* spins, int* cas, int* outer_sst) {
  if (!B || nget < 0 || chain0 < 0 || chain0 + nget > B->nchains || !offsets)
    return fail(CTHYB_ERR_ARG, "bad chain range or offsets");
  CK(cudaStreamSynchronize(B->stream));
  // segments of consecutive chains in one group
  struct Seg { GroupHost* G; int c0, i0, n; };
  std::vector<Seg> segs;
  for (int i = 0; i < nget; ++i) {
    GroupHost* G;
    int c;
    int rc = find_chain(B, chain0 + i, &G, &c);
    if (rc) return rc;
    if (segs.empty() || segs.back().G != G) segs.push_back(Seg{G, c, i, 0});
    segs.back().n++;
  }
  std::vector<int> cnt(nget), out(nget);
  int* d = nullptr;
  CK(cudaMalloc(&d, (size_t)(2 * nget + 2) * 4));
  cudaError_t e = cudaSuccess;
  for (const Seg& sg : segs) {
    if (e != cudaSuccess) break;
    k_get_configs<<<(sg.n + WPB - 1) / WPB, WPB * 32, 0, B->stream>>>(sg.G->g, sg.c0, sg.n, nullptr, d + sg.i0,
                                                                      d + nget + sg.i0, nullptr, nullptr);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(cnt.data(), d, (size_t)nget * 4, cudaMemcpyDeviceToHost, B->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(out.data(), d + nget, (size_t)nget * 4, cudaMemcpyDeviceToHost, B->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(B->stream);
  cudaFree(d);
  CK(e);
  offsets[0] = 0;
  for (int i = 0; i < nget; ++i) offsets[i + 1] = offsets[i] + cnt[i];
  if (outer_sst)
    for (int i = 0; i < nget; ++i) outer_sst[i] = out[i];
  if (!taus && !orbs && !spins && !cas) return CTHYB_OK;
  const int nop = offsets[nget];
  if (nop > cap) return fail(CTHYB_ERR_CAPACITY, "output arrays smaller than the operator count");
  if (nop == 0) return CTHYB_OK;
  std::vector<double> t(nop);
  std::vector<int> code(nop);
  char* db = nullptr;
  CK(cudaMalloc(&db, (size_t)nop * 12 + (size_t)(nget + 1) * 4 + 16));
  double* dt = (double*)db;
  int* dc = (int*)(db + (size_t)nop * 8);
  int* doffs = dc + nop;
  e = cudaMemcpyAsync(doffs, offsets, (size_t)(nget + 1) * 4, cudaMemcpyHostToDevice, B->stream);
  for (const Seg& sg : segs) {
    if (e != cudaSuccess) break;
    k_get_configs<<<(sg.n + WPB - 1) / WPB, WPB * 32, 0, B->stream>>>(sg.G->g, sg.c0, sg.n, doffs + sg.i0, nullptr,
                                                                      nullptr, dt, dc);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(t.data(), dt, (size_t)nop * 8, cudaMemcpyDeviceToHost, B->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(code.data(), dc, (size_t)nop * 4, cudaMemcpyDeviceToHost, B->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(B->stream);
  cudaFree(db);
  CK(e);
  for (int i = 0; i < nop; ++i) {
    if (taus) taus[i] = t[i];
    const int f = code[i] >> 1;
    if (orbs) orbs[i] = f / 2 + 1;
    if (spins) spins[i] = f % 2 + 1;
    if (cas) cas[i] = (code[i] & 1) + 1;
  }
  return CTHYB_OK;
}

int cthyb_batch_set_config(cthyb_batch_t B, int chain, int n, const double* taus, const int* orbs,
                           const int* spins, const int* cas, int outer_sst) {
  const int offs[2] = {0, n};
  return cthyb_batch_set_configs(B, chain, 1, offs, taus, orbs, spins, cas, &outer_sst);
}

// Whether any group of the batch has off-diagonal hybridisation (the
// per-flavour paths below -- set_mc_config, the LU refresh, gradients --
// do not apply to it).
static bool any_offdiag(cthyb_batch_t B) {
  for (const GroupHost& G : B->groups)
    if (G.g.offdiag) return true;
  return false;
}

int cthyb_batch_set_configs(cthyb_batch_t B, int chain0, int nset, const int* offsets, const double* taus,
                            const int* orbs, const int* spins, const int* cas, const int* outer_sst) {
  if (!B || nset < 0 || chain0 < 0 || chain0 + nset > B->nchains || !offsets || !outer_sst || offsets[0] != 0)
    return fail(CTHYB_ERR_ARG, "bad chain range or offsets");
  if (any_offdiag(B)) return fail(CTHYB_ERR_UNSUPPORTED, "set_mc_config with off-diagonal hybridisation");
  for (int i = 0; i < nset; ++i)
    if (offsets[i + 1] < offsets[i]) return fail(CTHYB_ERR_ARG, "offsets must not decrease");
  if (offsets[nset] > 0 && (!taus || !orbs || !spins || !cas)) return fail(CTHYB_ERR_ARG, "null operator arrays");
  // check every configuration before the first device write
  struct Seg { GroupHost* G; int c0, i0, n; std::vector<double> t; std::vector<int> code, offs, outer; };
  std::vector<Seg> segs;
  for (int i = 0; i < nset; ++i) {
    GroupHost* G;
    int c;
    int rc = find_chain(B, chain0 + i, &G, &c);
    if (rc) return rc;
    if (segs.empty() || segs.back().G != G) segs.push_back(Seg{G, c, i, 0, {}, {}, {0}, {}});
    Seg& sg = segs.back();
    const int o = offsets[i], n = offsets[i + 1] - offsets[i];
    rc = stage_config(B, G, n, taus + o, orbs + o, spins + o, cas + o, outer_sst[i], sg.t, sg.code);
    if (rc) return rc;
    sg.offs.push_back((int)sg.t.size());
    sg.outer.push_back(outer_sst[i]);
    sg.n++;
  }
  for (Seg& sg : segs) {
    int rc = upload_configs(B, sg.G, sg.c0, sg.n, sg.offs, sg.t, sg.code, sg.outer);
    if (rc) return rc;
  }
  return CTHYB_OK;
}

int cthyb_batch_minv(cthyb_batch_t B, int chain, int f, int* kout, double* out) {
  GroupHost* G;
  int c;
  int rc = find_chain(B, chain, &G, &c);
  if (rc) return rc;
  Hdr h;
  rc = read_hdr(B, G, c, h);
  if (rc) return rc;
  const int kcap = G->g.kcap, k = h.k[f];
  *kout = k;
  if (!out) return CTHYB_OK;
  char* base = G->g.base + (size_t)c * G->g.stride;
  std::vector<double> Mf((size_t)kcap * kcap);
  std::vector<short> sc(kcap), sa(kcap);
  CK(cudaMemcpy(Mf.data(), base + G->g.o_M + (size_t)f * kcap * kcap * 8, Mf.size() * 8, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(sc.data(), base + G->g.o_srt_slot + (size_t)(2 * f) * kcap * 2, kcap * 2, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(sa.data(), base + G->g.o_srt_slot + (size_t)(2 * f + 1) * kcap * 2, kcap * 2,
                cudaMemcpyDeviceToHost));
  for (int ra = 0; ra < k; ++ra)
    for (int rcn = 0; rcn < k; ++rcn) out[(size_t)ra * k + rcn] = Mf[(size_t)sa[ra] * kcap + sc[rcn]];
  return CTHYB_OK;
}

// Dense-block trace gradients of the chains of one group (directions of
// cthyb_model_set_directions) into device arrays gp (chains of the group x
// nparams) and lw[2c + 1], in chunks of chains that keep the stored kets
// within 2 GiB; enqueued on st (synchronises once for the largest bin).
static int dense_group_gradients(cthyb_batch_t B, GroupHost& G, int nparams, double* gp, double* lw,
                                 cudaStream_t st) {
  const HostModel& hm = B->model->hm;
  const int n = G.desc.nchains;
  int* d_mx = nullptr;
  CK(cudaMalloc(&d_mx, sizeof(int)));
  int mx = 0;
  cudaError_t e = cudaMemsetAsync(d_mx, 0, sizeof(int), st);
  if (e == cudaSuccess) {
    k_max_bin<<<(n + 127) / 128, 128, 0, st>>>(G.g, d_mx);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(&mx, d_mx, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  cudaFree(d_mx);
  const size_t ld = hm.nsmax;
  const size_t stride = align_up(((size_t)mx + 1) * (ld * ld + ld) + (size_t)mx + 2, 32);
  const int chunk = (int)std::max<size_t>(1, std::min<size_t>(n, ((size_t)2 << 30) / (stride * 8)));
  double* scr = nullptr;
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&scr, (size_t)chunk * stride * 8, st);
  for (int c0 = 0; c0 < n && e == cudaSuccess; c0 += chunk) {
    k_grad_dense<<<std::min(chunk, n - c0), 128, 0, st>>>(B->model->dm, G.g, c0, B->model->d_dir, nparams, gp, lw,
                                                          scr, stride, mx);
    e = cudaGetLastError();
  }
  if (scr) cudaFreeAsync(scr, st);
  if (e != cudaSuccess) return fail(CTHYB_ERR_CUDA, std::string("dense trace gradients: ") + cudaGetErrorString(e));
  return CTHYB_OK;
}

static bool any_dense(cthyb_batch_t B) {
  for (GroupHost& G : B->groups)
    if (G.g.o_chk) return true;
  return false;
}

int cthyb_batch_gradients(cthyb_batch_t B, int nparams, const double* dE, double* grad_delta, double* grad_params,
                          double* log_weights) {
  const bool dense = B && any_dense(B);
  if (!B || nparams < 0 || nparams > NPARMAX || (nparams > 0 && !grad_params) ||
      (nparams > 0 && !dense && !dE))
    return fail(CTHYB_ERR_ARG, "bad arguments (nparams must be 0..32)");
  if (any_offdiag(B)) return fail(CTHYB_ERR_UNSUPPORTED, "gradients with off-diagonal hybridisation");
  const HostModel& hm = B->model->hm;
  if (nparams > 0 && dense && (dE || B->model->ndir != nparams))
    return fail(CTHYB_ERR_ARG, "dense-block models: pass dE = NULL and set the directions with cthyb_model_set_directions");
  CK(cudaStreamSynchronize(B->stream));
  double* d_dE = nullptr;
  if (nparams > 0 && !dense) {
    CK(cudaMalloc(&d_dE, sizeof(double) * (size_t)nparams * hm.ns));
    CK(cudaMemcpy(d_dE, dE, sizeof(double) * (size_t)nparams * hm.ns, cudaMemcpyHostToDevice));
  }
  int rc = CTHYB_OK;
  for (GroupHost& G : B->groups) {
    const int n = G.desc.nchains, nft = G.g.nftau, nf = hm.nf;
    double *gd = nullptr, *gp = nullptr, *lw = nullptr;
    cudaError_t e = cudaMalloc(&gd, sizeof(double) * (size_t)n * nf * nft);
    if (e == cudaSuccess) e = cudaMalloc(&gp, sizeof(double) * (size_t)n * std::max(nparams, 1));
    if (e == cudaSuccess) e = cudaMalloc(&lw, sizeof(double) * (size_t)n * 2);
    if (e == cudaSuccess) e = cudaMemsetAsync(gd, 0, sizeof(double) * (size_t)n * nf * nft, B->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(lw, 0, sizeof(double) * (size_t)n * 2, B->stream);
    if (e == cudaSuccess) {
      k_grad<<<(n + WPB - 1) / WPB, WPB * 32, 0, B->stream>>>(B->model->dm, G.g, d_dE, dense ? 0 : nparams, gd, gp,
                                                              lw);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess && dense && nparams > 0) {
      const int rc2 = dense_group_gradients(B, G, nparams, gp, lw, B->stream);
      if (rc2) {
        cudaFree(gd);
        cudaFree(gp);
        cudaFree(lw);
        if (d_dE) cudaFree(d_dE);
        return rc2;
      }
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(B->stream);
    if (e == cudaSuccess) {
      std::vector<double> h((size_t)n * nf * nft);
      e = cudaMemcpy(h.data(), gd, h.size() * 8, cudaMemcpyDeviceToHost);
      // per chain (Nd, 2, Nftau) Fortran order
      if (e == cudaSuccess && grad_delta)
        for (int ch = 0; ch < n; ++ch)
          for (int f = 0; f < nf; ++f)
            for (int j = 0; j < nft; ++j)
              grad_delta[(size_t)(G.chain0 + ch) * nf * nft + (f / 2) + hm.nd * ((f % 2) + 2 * (size_t)j)] =
                  h[((size_t)ch * nf + f) * nft + j];
    }
    if (e == cudaSuccess && nparams > 0)
      e = cudaMemcpy(grad_params + (size_t)G.chain0 * nparams, gp, sizeof(double) * (size_t)n * nparams,
                     cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && log_weights)
      e = cudaMemcpy(log_weights + (size_t)G.chain0 * 2, lw, sizeof(double) * (size_t)n * 2, cudaMemcpyDeviceToHost);
    cudaFree(gd);
    cudaFree(gp);
    cudaFree(lw);
    if (e != cudaSuccess) {
      rc = fail(CTHYB_ERR_CUDA, std::string("gradients: ") + cudaGetErrorString(e));
      break;
    }
  }
  if (d_dE) cudaFree(d_dE);
  return rc;
}

int cthyb_batch_gradients_device(cthyb_batch_t B, int nparams, const double* dE_dev, double* grad_delta_dev,
                                 double* grad_params_dev, double* log_weights_dev, void* stream) {
  const bool dense = B && any_dense(B);
  if (!B || nparams < 0 || nparams > NPARMAX || !grad_delta_dev || !log_weights_dev ||
      (nparams > 0 && (!grad_params_dev || (!dense && !dE_dev))))
    return fail(CTHYB_ERR_ARG, "bad arguments (nparams must be 0..32)");
  if (any_offdiag(B)) return fail(CTHYB_ERR_UNSUPPORTED, "gradients with off-diagonal hybridisation");
  if (nparams > 0 && dense && (dE_dev || B->model->ndir != nparams))
    return fail(CTHYB_ERR_ARG, "dense-block models: pass dE = NULL and set the directions with cthyb_model_set_directions");
  const int nft = B->groups[0].g.nftau, nf = B->model->hm.nf;
  for (GroupHost& G : B->groups)
    if (G.g.nftau != nft) return fail(CTHYB_ERR_ARG, "gradients need one Nftau for all groups");
  cudaStream_t st = stream ? (cudaStream_t)stream : B->stream;
  if (st != B->stream) {  // order after the batch's queued sweeps
    cudaEvent_t ev;
    CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    CK(cudaEventRecord(ev, B->stream));
    CK(cudaStreamWaitEvent(st, ev, 0));
    CK(cudaEventDestroy(ev));
  }
  CK(cudaMemsetAsync(grad_delta_dev, 0, sizeof(double) * (size_t)B->nchains * nf * nft, st));
  for (GroupHost& G : B->groups) {
    const int n = G.desc.nchains;
    k_grad<<<(n + WPB - 1) / WPB, WPB * 32, 0, st>>>(B->model->dm, G.g, dE_dev, dense ? 0 : nparams,
                                                     grad_delta_dev + (size_t)G.chain0 * nf * nft,
                                                     grad_params_dev ? grad_params_dev + (size_t)G.chain0 * nparams
                                                                     : nullptr,
                                                     log_weights_dev + (size_t)G.chain0 * 2);
    CK(cudaGetLastError());
    if (dense && nparams > 0) {
      const int rc = dense_group_gradients(B, G, nparams, grad_params_dev + (size_t)G.chain0 * nparams,
                                           log_weights_dev + (size_t)G.chain0 * 2, st);
      if (rc) return rc;
    }
  }
  return CTHYB_OK;
}

int cthyb_batch_refresh_minv(cthyb_batch_t B, int replace, double* maxdev) {
  if (!B) return fail(CTHYB_ERR_ARG, "null");
  if (any_offdiag(B)) return fail(CTHYB_ERR_UNSUPPORTED, "LU refresh with off-diagonal hybridisation");
  CK(cudaMemsetAsync(B->d_dev, 0, sizeof(double), B->stream));
  for (GroupHost& G : B->groups) {
    if (2 * G.g.kcap * G.g.kcap > 2 * B->model->hm.nsmax * B->model->hm.nsmax &&
        (size_t)2 * G.g.kcap * G.g.kcap * 8 > G.g.o_log - G.g.o_dense)
      return fail(CTHYB_ERR_INTERNAL, "refresh scratch too small");
    int nblk = (G.desc.nchains + WPB - 1) / WPB;
    k_refresh<<<nblk, WPB * 32, 0, B->stream>>>(B->model->dm, G.g, replace, B->d_dev);
    CK(cudaGetLastError());
  }
  double d = 0;
  CK(cudaMemcpyAsync(&d, B->d_dev, sizeof(double), cudaMemcpyDeviceToHost, B->stream));
  CK(cudaStreamSynchronize(B->stream));
  if (maxdev) *maxdev = d;
  return CTHYB_OK;
}

int cthyb_batch_log_weights_device(cthyb_batch_t B, double* lw_dev, void* stream) {
  if (!B || !lw_dev) return fail(CTHYB_ERR_ARG, "null");
  cudaStream_t st = stream ? (cudaStream_t)stream : B->stream;
  if (st != B->stream) {  // after the batch's queued work
    cudaEvent_t ev;
    CK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    cudaError_t e = cudaEventRecord(ev, B->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(st, ev, 0);
    cudaEventDestroy(ev);
    CK(e);
  }
  for (GroupHost& G : B->groups) {
    k_log_weights<<<(G.desc.nchains + 127) / 128, 128, 0, st>>>(B->model->dm, G.g, lw_dev);
    CK(cudaGetLastError());
  }
  return CTHYB_OK;
}

int cthyb_batch_chain_stats(cthyb_batch_t B, int group, double* out) {
  if (!B || !out || group < 0 || group >= (int)B->groups.size()) return fail(CTHYB_ERR_ARG, "bad arguments");
  GroupHost& G = B->groups[group];
  const int n = G.desc.nchains;
  double* d = nullptr;
  CK(cudaMallocAsync((void**)&d, (size_t)4 * n * sizeof(double), B->stream));
  k_chain_stats<<<(n + 127) / 128, 128, 0, B->stream>>>(G.g, d);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, d, (size_t)4 * n * sizeof(double), cudaMemcpyDeviceToHost, B->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(B->stream);
  cudaFreeAsync(d, B->stream);
  CK(e);
  return CTHYB_OK;
}

int cthyb_batch_group_gtau_raw(cthyb_batch_t B, int group, double* out) {
  if (!B || !out || group < 0 || group >= (int)B->groups.size()) return fail(CTHYB_ERR_ARG, "bad arguments");
  GroupHost& G = B->groups[group];
  const size_t row = (size_t)B->model->hm.nf * G.g.ntau * sizeof(double);
  CK(cudaMemcpy2DAsync(out, row, G.g.base + G.g.o_gtau, G.g.stride, row, G.desc.nchains, cudaMemcpyDeviceToHost,
                       B->stream));
  CK(cudaStreamSynchronize(B->stream));
  return CTHYB_OK;
}

int cthyb_batch_drift(cthyb_batch_t B, double* max_dev_m, double* max_dev_logdet, int64_t* refreshes,
                      int64_t* sign_errors, int reset) {
  if (!B) return fail(CTHYB_ERR_ARG, "null");
  unsigned long long* d = nullptr;
  CK(cudaMallocAsync((void**)&d, 4 * sizeof(unsigned long long), B->stream));
  cudaError_t e = cudaMemsetAsync(d, 0, 4 * sizeof(unsigned long long), B->stream);
  for (GroupHost& G : B->groups) {
    if (e != cudaSuccess) break;
    k_drift<<<(G.desc.nchains + 127) / 128, 128, 0, B->stream>>>(G.g, d, reset);
    e = cudaGetLastError();
  }
  unsigned long long hbuf[4] = {0, 0, 0, 0};
  if (e == cudaSuccess) e = cudaMemcpyAsync(hbuf, d, sizeof(hbuf), cudaMemcpyDeviceToHost, B->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(B->stream);
  cudaFreeAsync(d, B->stream);
  CK(e);
  double v;
  if (max_dev_m) {
    std::memcpy(&v, &hbuf[0], 8);
    *max_dev_m = v;
  }
  if (max_dev_logdet) {
    std::memcpy(&v, &hbuf[1], 8);
    *max_dev_logdet = v;
  }
  if (refreshes) *refreshes = (int64_t)hbuf[2];
  if (sign_errors) *sign_errors = (int64_t)hbuf[3];
  return CTHYB_OK;
}

int cthyb_batch_set_log(cthyb_batch_t B, int64_t cap) {
  if (!B || cap < 0) return fail(CTHYB_ERR_ARG, "bad arguments");
  // re-layout is only possible right after creation: the log area is the
  // last region of each chain block, so grow the slab by copying chains.
  CK(cudaStreamSynchronize(B->stream));
  std::vector<DGroup> oldg;
  for (GroupHost& G : B->groups) oldg.push_back(G.g);
  size_t total = 0;
  for (GroupHost& G : B->groups) {
    DGroup save = G.g;
    layout_group(B, G, cap);
    G.g.base = save.base;
    G.g.hybr = save.hybr;
    G.g.hybr_full = save.hybr_full;
    G.g.empty_w = save.empty_w;
    G.g.err_flag = save.err_flag;
    G.g.edges = save.edges;
    G.g.ekeys = save.ekeys;
    G.g.score_dE = save.score_dE;
    G.g.nsym = save.nsym;
    G.g.symmoves = save.symmoves;
    total += (size_t)G.desc.nchains * G.g.stride;
  }
  char* slab = nullptr;
  CK(slab_alloc(&slab, total, B->stream));
  CK(cudaMemsetAsync(slab, 0, total, B->stream));
  CK(cudaStreamSynchronize(B->stream));
  size_t off = 0;
  for (size_t gi = 0; gi < B->groups.size(); ++gi) {
    GroupHost& G = B->groups[gi];
    char* nb = slab + off;
    size_t keep = std::min(oldg[gi].o_log, G.g.o_log);
    for (int c = 0; c < G.desc.nchains; ++c)
      CK(cudaMemcpy(nb + (size_t)c * G.g.stride, oldg[gi].base + (size_t)c * oldg[gi].stride, keep,
                    cudaMemcpyDeviceToDevice));
    G.g.base = nb;
    off += (size_t)G.desc.nchains * G.g.stride;
    // reset the per-chain log counters
    for (int c = 0; c < G.desc.nchains; ++c) {
      Hdr h;
      CK(cudaMemcpy(&h, nb + (size_t)c * G.g.stride + G.g.o_hdr, sizeof(Hdr), cudaMemcpyDeviceToHost));
      h.logn = 0;
      h.kv = -1;  // regions after the log (checkpoints, scratch) start empty
      h.bv = (1 << G.g.L) + 1;
      CK(cudaMemcpy(nb + (size_t)c * G.g.stride + G.g.o_hdr, &h, sizeof(Hdr), cudaMemcpyHostToDevice));
    }
  }
  slab_free(B->slab, B->stream);
  B->slab = slab;
  B->logcap = cap;
  return upload_groups(B);
}

int cthyb_batch_get_log(cthyb_batch_t B, int chain, void* rec, int64_t* n) {
  GroupHost* G;
  int c;
  int rc = find_chain(B, chain, &G, &c);
  if (rc) return rc;
  Hdr h;
  rc = read_hdr(B, G, c, h);
  if (rc) return rc;
  long long m = std::min<long long>(h.logn, G->g.logcap);
  *n = h.logn;
  if (rec && m > 0)
    CK(cudaMemcpy(rec, G->g.base + (size_t)c * G->g.stride + G->g.o_log, (size_t)m * sizeof(cthyb_record),
                  cudaMemcpyDeviceToHost));
  return CTHYB_OK;
}

// Phase cycle counters (builds with -DCTHYB_PROFILE), summed over chains.
int cthyb_debug_phase_cycles(cthyb_batch_t B, int64_t* out10) {
  if (!B || !out10) return fail(CTHYB_ERR_ARG, "null");
  CK(cudaStreamSynchronize(B->stream));
  for (int i = 0; i < 10; ++i) out10[i] = 0;
  for (GroupHost& G : B->groups)
    for (int c = 0; c < G.desc.nchains; ++c) {
      Hdr h;
      CK(cudaMemcpy(&h, G.g.base + (size_t)c * G.g.stride + G.g.o_hdr, sizeof(Hdr), cudaMemcpyDeviceToHost));
      for (int i = 0; i < 10; ++i) out10[i] += h.prof[i];
    }
  return CTHYB_OK;
}

int cthyb_batch_results_full(cthyb_batch_t B, int chain, double* gtau_full) {
  GroupHost* G;
  int c;
  int rc = find_chain(B, chain, &G, &c);
  if (rc) return rc;
  if (!G->g.offdiag) return fail(CTHYB_ERR_ARG, "not an off-diagonal group");
  if (!gtau_full) return fail(CTHYB_ERR_ARG, "null");
  Hdr h;
  rc = read_hdr(B, G, c, h);
  if (rc) return rc;
  const int nf = B->model->hm.nf, nt = G->g.ntau;
  std::vector<double> acc((size_t)nf * nf * nt);
  CK(cudaMemcpy(acc.data(), G->g.base + (size_t)c * G->g.stride + G->g.o_gfull, acc.size() * 8,
                cudaMemcpyDeviceToHost));
  const double ms = h.cnt_meas ? h.meas_sign / (double)h.cnt_meas : 0.0;
  const double scale = (h.cnt_meas && ms != 0.0) ? (double)nt / (G->g.beta * G->g.beta) / ((double)h.cnt_meas * ms) : 0.0;
  for (size_t i = 0; i < acc.size(); ++i) gtau_full[i] = acc[i] * scale;  // -acc * zScaling * Ntau / beta^2
  return CTHYB_OK;
}

int cthyb_batch_results_accpair(cthyb_batch_t B, int chain, double* accpair) {
  GroupHost* G;
  int c;
  int rc = find_chain(B, chain, &G, &c);
  if (rc) return rc;
  if (!G->g.o_accpair) return fail(CTHYB_ERR_ARG, "the group does not measure accepted pairs (CTHYB_FLAG_ACCPAIR)");
  if (!accpair) return fail(CTHYB_ERR_ARG, "null");
  const int nf = B->model->hm.nf, nt = G->g.ntau, nd = B->model->hm.nd;
  std::vector<double> raw((size_t)nf * nt);
  CK(cudaMemcpy(raw.data(), G->g.base + (size_t)c * G->g.stride + G->g.o_accpair, raw.size() * 8,
                cudaMemcpyDeviceToHost));
  for (int f = 0; f < nf; ++f)
    for (int t = 0; t < nt; ++t) accpair[(f / 2) + nd * ((f % 2) + 2 * (size_t)t)] = raw[(size_t)f * nt + t];
  return CTHYB_OK;
}

int cthyb_batch_results_gleg_full(cthyb_batch_t B, int chain, double* gleg_full) {
  GroupHost* G;
  int c;
  int rc = find_chain(B, chain, &G, &c);
  if (rc) return rc;
  if (!G->g.offdiag) return fail(CTHYB_ERR_ARG, "not an off-diagonal group");
  if (!gleg_full) return fail(CTHYB_ERR_ARG, "null");
  const int nf = B->model->hm.nf, nleg = G->g.nleg;
  if (nleg <= 0) return CTHYB_OK;
  Hdr h;
  rc = read_hdr(B, G, c, h);
  if (rc) return rc;
  std::vector<double> raw((size_t)nf * nf * nleg);
  CK(cudaMemcpy(raw.data(), G->g.base + (size_t)c * G->g.stride + G->g.o_gleg, raw.size() * 8,
                cudaMemcpyDeviceToHost));
  const double cnt = (double)h.cnt_meas, ms = h.cnt_meas ? h.meas_sign / cnt : 0.0;
  const double zs = h.cnt_meas ? -1.0 / (cnt * ms) : 0.0;
  // GLeg_full * sqrt(2l+1)/beta, then -GLeg_full * zScaling (CTQMC.F90:8766-8771)
  for (size_t i = 0; i < raw.size(); ++i)
    gleg_full[i] = -(raw[i] * std::sqrt(2.0 * (double)(i % nleg) + 1.0) / G->g.beta) * zs;
  return CTHYB_OK;
}

int cthyb_batch_minv_full(cthyb_batch_t B, int chain, int* kout, double* out) {
  GroupHost* G;
  int c;
  int rc = find_chain(B, chain, &G, &c);
  if (rc) return rc;
  if (!G->g.offdiag || !kout) return fail(CTHYB_ERR_ARG, "not an off-diagonal group");
  Hdr h;
  rc = read_hdr(B, G, c, h);
  if (rc) return rc;
  const int k = h.K / 2, ld = G->g.kcap;
  *kout = k;
  if (!out || k == 0) return CTHYB_OK;
  std::vector<double> M((size_t)ld * k);
  CK(cudaMemcpy(M.data(), G->g.base + (size_t)c * G->g.stride + G->g.o_M, M.size() * 8, cudaMemcpyDeviceToHost));
  for (int j = 0; j < k; ++j)
    for (int i = 0; i < k; ++i) out[(size_t)j * k + i] = M[(size_t)j * ld + i];
  return CTHYB_OK;
}

int cthyb_batch_move_counters4(cthyb_batch_t B, int chain, int64_t* out4) {
  if (!out4) return fail(CTHYB_ERR_ARG, "null");
  GroupHost* G;
  int lc;
  int rc = find_chain(B, chain, &G, &lc);
  if (rc) return rc;
  Hdr h;
  rc = read_hdr(B, G, lc, h);
  if (rc) return rc;
  out4[0] = h.try_add4;
  out4[1] = h.acc_add4;
  out4[2] = h.try_rem4;
  out4[3] = h.acc_rem4;
  return CTHYB_OK;
}

int cthyb_batch_move_counters(cthyb_batch_t B, int chain, int64_t* out5) {
  if (!out5) return fail(CTHYB_ERR_ARG, "null");
  GroupHost* G;
  int lc;
  int rc = find_chain(B, chain, &G, &lc);
  if (rc) return rc;
  Hdr h;
  rc = read_hdr(B, G, lc, h);
  if (rc) return rc;
  out5[0] = h.try_glob;
  out5[1] = h.acc_glob;
  out5[2] = h.qn_glob;
  out5[3] = h.try_shift;
  out5[4] = h.acc_shift;
  return CTHYB_OK;
}

int cthyb_batch_work_counters(cthyb_batch_t B, int64_t* out8, int reset) {
  if (!B || !out8) return fail(CTHYB_ERR_ARG, "null");
  CK(cudaStreamSynchronize(B->stream));
  for (int i = 0; i < 8; ++i) out8[i] = 0;
  for (GroupHost& G : B->groups)
    for (int c = 0; c < G.desc.nchains; ++c) {
      char* p = G.g.base + (size_t)c * G.g.stride + G.g.o_hdr;
      Hdr h;
      CK(cudaMemcpy(&h, p, sizeof(Hdr), cudaMemcpyDeviceToHost));
      out8[0] += h.w_mbytes;
      out8[1] += h.w_mflops;
      out8[2] += h.w_opbytes;
      out8[3] += h.w_nodes;
      out8[4] += h.try_add + h.try_rem;
      out8[5] += h.acc_add + h.acc_rem;
      out8[6] += h.w_tflops;
      out8[7] += h.w_tbytes;
      if (reset) {
        h.w_mbytes = h.w_mflops = h.w_opbytes = h.w_nodes = h.w_tflops = h.w_tbytes = 0;
        CK(cudaMemcpy(p, &h, sizeof(Hdr), cudaMemcpyHostToDevice));
      }
    }
  return CTHYB_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// FP64 peak of the running device, the denominator of the FP64 rooflines:
// independent fused multiply-adds on the CUDA cores (eight chains a
// thread) and m8n8k4 FP64 tensor-core MMAs (four accumulators a warp), each
// over a grid of 8 blocks of 256 threads per multiprocessor.  Every thread
// writes one double of `out` (grid x block entries).
namespace cthyb {
__global__ void __launch_bounds__(256) k_peak_dfma(double* out, int iters, double a, double b) {
  double x[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) x[j] = threadIdx.x * 1e-9 + j;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 8; ++j) x[j] = fma(x[j], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int j = 0; j < 8; ++j) s += x[j];
  out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}
__global__ void __launch_bounds__(256) k_peak_dmma(double* out, int iters, double a, double b) {
  double c[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) c[j] = threadIdx.x * 1e-9 + j;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 4; ++j) dmma_884(c[2 * j], c[2 * j + 1], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int j = 0; j < 8; ++j) s += c[j];
  out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}
}  // namespace cthyb

extern "C" int cthyb_probe_fp64(double* dfma_gflops, double* dmma_gflops) {
  using namespace cthyb;
  int dev = 0, nsm = 0;
  CK(cudaGetDevice(&dev));
  CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  const int block = 256, grid = 8 * nsm, iters = 4096;
  double* out = nullptr;
  CK(cudaMalloc(&out, sizeof(double) * (size_t)grid * block));
  cudaEvent_t e0, e1;
  cudaError_t e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  float best[2] = {3.4e38f, 3.4e38f};
  for (int rep = 0; rep < 3 && e == cudaSuccess; ++rep)
    for (int kind = 0; kind < 2 && e == cudaSuccess; ++kind) {
      cudaEventRecord(e0);
      if (kind == 0) k_peak_dfma<<<grid, block>>>(out, iters, 0.999, 1e-3);
      else k_peak_dmma<<<grid, block>>>(out, iters, 0.999, 1e-3);
      cudaEventRecord(e1);
      e = cudaEventSynchronize(e1);
      float ms = 0.f;
      if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
      if (ms < best[kind]) best[kind] = ms;
    }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  CK(e);
  const double threads = (double)grid * block;
  // DFMA: 8 FMAs a thread and iteration; DMMA: 4 MMAs of 8x8x4 FMAs a warp
  if (dfma_gflops) *dfma_gflops = 2.0 * 8 * iters * threads / (best[0] * 1e6);
  if (dmma_gflops) *dmma_gflops = 2.0 * 256 * 4 * iters * (threads / 32) / (best[1] * 1e6);
  return CTHYB_OK;
}

// ---------------------------------------------------------------------------
// Allocation-free inverse hybridisation matrix.
//
// For callers that cannot call cudaMalloc -- a host already running inside a
// fixed device-memory budget (a Fortran solver whose arrays were sized at
// start-up, a process that hands all device memory to another framework's
// caching allocator, or code that must not allocate between the capture and
// the replay of its own work).  The two k x k work matrices of the
// elimination live in one file-scope device array instead of in a chain
// slab, so every GPU that loads this library holds it until the process
// exits.  All calls share it: calls whose kernels overlap on the GPU race on
// it, and it keeps the last call's contents (every call writes the full
// k x k region it reads, so nothing stale is ever used).
namespace cthyb {
constexpr int NOALLOC_KMAX = 256;  // largest k accepted (2 * 256^2 doubles = 1 MiB)
static __device__ __align__(256) double g_noalloc_scratch[2 * NOALLOC_KMAX * NOALLOC_KMAX];

// One warp: H(a, c) = F(tau_a - tau_c) by the linear interpolation of
// get_HybrF (Trace.F90:1014-1033; grid coordinate tau * ((Nftau - 1) / beta),
// equal to the reference's tau / beta * (Nftau - 1) to within rounding),
// Gauss-Jordan elimination with partial
// pivoting on [H | 1] in the scratch array, M = H^{-1} written with rows =
// creators and columns = annihilators, log|det H| and its sign.
__global__ void k_minv_noalloc(double* scratch, int k, const double* __restrict__ tau_c,
                               const double* __restrict__ tau_a, const double* __restrict__ F, int nftau,
                               double beta, double* __restrict__ minv, double* __restrict__ logdet) {
  const int lane = threadIdx.x & 31;
  const int ld = k;
  double* H = scratch;
  double* I = scratch + (size_t)k * k;
  const double hs = (double)(nftau - 1) / beta;
  for (int e = lane; e < k * k; e += 32) {
    int ia = e % k, ic = e / k;
    double tau = tau_a[ia] - tau_c[ic];
    double sig = 1.0;
    if (tau < 0.0) {
      tau += beta;
      sig = -1.0;
    }
    double n = tau * hs;
    int in = (int)n;
    int i = min(max(in, 0), nftau - 2);
    H[(size_t)ic * ld + ia] = sig * (F[i] + (n - (double)in) * (F[i + 1] - F[i]));
    I[(size_t)ic * ld + ia] = (ia == ic) ? 1.0 : 0.0;
  }
  __syncwarp();
  double dlog = 0.0, dsign = 1.0;
  for (int j = 0; j < k; ++j) {
    double best = -1.0;
    int bi = j;
    for (int i = j + lane; i < k; i += 32) {
      double a = fabs(H[(size_t)j * ld + i]);
      if (a > best) {
        best = a;
        bi = i;
      }
    }
    for (int o = 16; o; o >>= 1) {
      double ob = __shfl_xor_sync(FULL, best, o);
      int oi = __shfl_xor_sync(FULL, bi, o);
      if (ob > best || (ob == best && oi < bi)) {
        best = ob;
        bi = oi;
      }
    }
    if (best <= 0.0) {  // singular
      if (lane == 0) {
        logdet[0] = -DHUGE;
        logdet[1] = 0.0;
      }
      return;
    }
    if (bi != j) {
      for (int col = lane; col < k; col += 32) {
        double t = H[(size_t)col * ld + j];
        H[(size_t)col * ld + j] = H[(size_t)col * ld + bi];
        H[(size_t)col * ld + bi] = t;
        t = I[(size_t)col * ld + j];
        I[(size_t)col * ld + j] = I[(size_t)col * ld + bi];
        I[(size_t)col * ld + bi] = t;
      }
      dsign = -dsign;
    }
    __syncwarp();
    double piv = H[(size_t)j * ld + j];
    dlog += log(fabs(piv));
    if (piv < 0) dsign = -dsign;
    double ip = 1.0 / piv;
    for (int col = lane; col < k; col += 32) {
      H[(size_t)col * ld + j] *= ip;
      I[(size_t)col * ld + j] *= ip;
    }
    __syncwarp();
    for (int col = 0; col < k; ++col) {
      if (col == j) continue;
      double hj = H[(size_t)col * ld + j];
      double ij = I[(size_t)col * ld + j];
      for (int i = lane; i < k; i += 32) {
        if (i == j) continue;
        double fct = H[(size_t)j * ld + i];
        H[(size_t)col * ld + i] -= fct * hj;
        I[(size_t)col * ld + i] -= fct * ij;
      }
    }
    __syncwarp();
    for (int i = lane; i < k; i += 32)
      if (i != j) {
        I[(size_t)j * ld + i] -= H[(size_t)j * ld + i] * I[(size_t)j * ld + j];
        H[(size_t)j * ld + i] = 0.0;
      }
    __syncwarp();
  }
  // I(c, a) = H^{-1}: column-major k x k, rows creators, columns annihilators
  for (int e = lane; e < k * k; e += 32) minv[e] = I[e];
  if (lane == 0) {
    logdet[0] = dlog;
    logdet[1] = dsign;
  }
}

namespace {
std::mutex g_noalloc_mu;
double* g_noalloc_ptr[64] = {nullptr};
}  // namespace
}  // namespace cthyb

extern "C" {

// Allocation-free variant of the M rebuild (no counterpart in the
// reference): see include/cthyb_gpu.h.  The first call on a device looks up
// the device address of the scratch array with that device current (do it
// before any stream capture); later calls on that device only launch.
int cthyb_minv_rebuild_noalloc(int k, const double* tau_c, const double* tau_a, const double* ftau,
                               int nftau, double beta, double* minv, double* logdet, void* stream) {
  using namespace cthyb;
  if (k < 0 || k > NOALLOC_KMAX)
    return fail(CTHYB_ERR_CAPACITY, "cthyb_minv_rebuild_noalloc: k = " + std::to_string(k) +
                                        " exceeds the static scratch limit of " +
                                        std::to_string(NOALLOC_KMAX) + " operators per type");
  if (nftau < 2 || !(beta > 0.0) || !logdet || (k > 0 && (!tau_c || !tau_a || !ftau || !minv)))
    return fail(CTHYB_ERR_ARG, "cthyb_minv_rebuild_noalloc: bad arguments");
  int dev = 0;
  CK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return fail(CTHYB_ERR_ARG, "cthyb_minv_rebuild_noalloc: device ordinal out of range");
  double* scratch = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
      void* p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess)
        return fail(CTHYB_ERR_CUDA, std::string("cthyb_minv_rebuild_noalloc: cudaGetSymbolAddress: ") +
                                        cudaGetErrorString(e));
      g_noalloc_ptr[dev] = (double*)p;
    }
    scratch = g_noalloc_ptr[dev];
  }
  k_minv_noalloc<<<1, 32, 0, (cudaStream_t)stream>>>(scratch, k, tau_c, tau_a, ftau, nftau, beta, minv, logdet);
  CK(cudaGetLastError());
  return CTHYB_OK;
}

}  // extern "C"
