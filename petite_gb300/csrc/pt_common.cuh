// pt_common.cuh -- constants, random streams and arithmetic helpers shared by
// the shower kernels.  sm_103a only.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace pt {

// ---------------------------------------------------------------- constants
// Same expressions as PETITE's physical_constants.py:11-38, so every value
// rounds exactly as the Python module's does.
constexpr double kPi = 3.141592653589793;
constexpr double kMeV = 1e-3;
constexpr double kkeV = 1e-6;
constexpr double kAlpha = 1 / 137.035999;
constexpr double kMe = 510.998950 * kkeV;
constexpr double kMmu = 105.6583755 * kMeV;
constexpr double kCmToM = 0.01;
constexpr double kHbarc = 0.1973269804E-13;       // GeV cm
constexpr double kNAvogadro = 6.0221409e+23;

// ------------------------------------------------------------ random stream
// Philox4x32-10 (Salmon et al., SC'11).  Counter = (draw block lo, hi,
// particle key lo, hi), key = 64-bit seed.  Draw n of a particle uses block
// n>>1 and 64-bit half n&1; uniform double = (u64 >> 11) * 2^-53 in [0,1).
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
    const uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
    c = make_uint4(hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0);
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return c;
}

// The same Philox4x32-10 with the key schedule of a fixed seed precomputed
// (round r uses seed words + r * (0x9E3779B9, 0xBB67AE85)).  Kernels pass the
// table as a by-value parameter, so each round key is an operand read from
// the parameter space instead of two additions per round, and each round's
// two products are single 32x32->64 multiplies.
struct PhiloxRK {
  uint32_t k[20];
};
__host__ __device__ inline PhiloxRK philox_round_keys(uint64_t seed) {
  PhiloxRK R;
  uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
  for (int r = 0; r < 10; ++r) {
    R.k[2 * r] = k0;
    R.k[2 * r + 1] = k1;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return R;
}
__device__ __forceinline__ uint4 philox_rk(uint4 c, const PhiloxRK& R) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c.x;
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c.z;
    c = make_uint4((uint32_t)(p1 >> 32) ^ c.y ^ R.k[2 * r], (uint32_t)p1, (uint32_t)(p0 >> 32) ^ c.w ^ R.k[2 * r + 1],
                   (uint32_t)p0);
  }
  return c;
}

__host__ __device__ __forceinline__ uint64_t mix64(uint64_t z) {   // SplitMix64 finaliser
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__host__ __device__ __forceinline__ uint64_t primary_key(uint64_t i) { return mix64(i + 1); }
__host__ __device__ __forceinline__ uint64_t daughter_key(uint64_t parent, int bit) {
  return mix64(parent + 0x9E3779B97F4A7C15ull * (uint64_t)(1 + bit));
}

struct Rng {
  uint32_t s0, s1, k0, k1;   // seed lo/hi, particle key lo/hi
  uint64_t n;                // next draw index
  uint64_t spare;            // odd half of the current block
  __device__ __forceinline__ void init(uint64_t seed, uint64_t key) {
    s0 = (uint32_t)seed; s1 = (uint32_t)(seed >> 32);
    k0 = (uint32_t)key;  k1 = (uint32_t)(key >> 32);
    n = 0; spare = 0;
  }
  __device__ __forceinline__ uint64_t next_u64() {
    if (n & 1ull) { ++n; return spare; }
    const uint64_t blk = n >> 1;
    const uint4 o = philox4x32_10(make_uint4((uint32_t)blk, (uint32_t)(blk >> 32), k0, k1), s0, s1);
    spare = (uint64_t)o.z | ((uint64_t)o.w << 32);
    ++n;
    return (uint64_t)o.x | ((uint64_t)o.y << 32);
  }
  // Positions the stream at draw m (the odd half of a block is regenerated).
  __device__ __forceinline__ void seek(uint64_t m) {
    n = m;
    if (m & 1ull) {
      const uint64_t blk = m >> 1;
      const uint4 o = philox4x32_10(make_uint4((uint32_t)blk, (uint32_t)(blk >> 32), k0, k1), s0, s1);
      spare = (uint64_t)o.z | ((uint64_t)o.w << 32);
    }
  }
  __device__ __forceinline__ double u() { return (double)(next_u64() >> 11) * 0x1p-53; }
  // float form of the same draw (its top 24 bits); used by the float32 sampler.
  // Converted from a 32-bit integer: 64-bit conversions run on the FP64 pipe.
  __device__ __forceinline__ float uf() {
    const uint32_t hi = (uint32_t)(next_u64() >> 32);
    return __uint2float_rn(hi >> 8) * 0x1p-24f;
  }
  // uf() with the precomputed round keys of this stream's seed
  __device__ __forceinline__ float uf(const PhiloxRK& R) {
    uint64_t v;
    if (n & 1ull) {
      v = spare;
    } else {
      const uint64_t blk = n >> 1;
      const uint4 o = philox_rk(make_uint4((uint32_t)blk, (uint32_t)(blk >> 32), k0, k1), R);
      spare = (uint64_t)o.z | ((uint64_t)o.w << 32);
      v = (uint64_t)o.x | ((uint64_t)o.y << 32);
    }
    ++n;
    return __uint2float_rn((uint32_t)(v >> 32) >> 8) * 0x1p-24f;
  }
  // The float forms of the next D draws with a fixed number of Philox blocks,
  // (D+1)/2, whatever the stream's parity: a warp whose lanes sit at
  // different parities issues (D+1)/2 blocks instead of one per draw (the
  // branch of next_u64 diverges).  The same draws as D calls of uf().
  template <int D>
  __device__ __forceinline__ void take(float (&u)[D], const PhiloxRK& R) {
    constexpr int NB = (D + 1) / 2;
    constexpr int KS = (D & 1) ? (D - 1) / 2 : D / 2 - 1;   // block holding the odd half left over
    const bool odd = (n & 1ull) != 0;
    const uint64_t b0 = (n + 1) >> 1;                      // first block not yet drawn from
    uint32_t h[2 * NB];
    uint64_t left = 0;
#pragma unroll
    for (int k = 0; k < NB; ++k) {
      const uint64_t blk = b0 + (uint64_t)k;
      const uint4 o = philox_rk(make_uint4((uint32_t)blk, (uint32_t)(blk >> 32), k0, k1), R);
      h[2 * k] = o.y;
      h[2 * k + 1] = o.w;
      if (k == KS) left = (uint64_t)o.z | ((uint64_t)o.w << 32);
    }
    const uint32_t sp = (uint32_t)(spare >> 32);
#pragma unroll
    for (int j = 0; j < D; ++j) {
      const uint32_t w = odd ? (j == 0 ? sp : h[j > 0 ? j - 1 : 0]) : h[j];
      u[j] = __uint2float_rn(w >> 8) * 0x1p-24f;
    }
    n += D;
    if (n & 1ull) spare = left;      // only the parity that ends inside block KS gets here
  }

  // Look-ahead form for the float32 kernels: peek computes the float forms of
  // the next D draws ((D+1)/2 blocks, as take does) without consuming them;
  // advance then consumes the first `used` (0..D).  Only the odd halves' high
  // words are kept for the leftover, so after advance only uf()/take()/peek()
  // may follow (not u()).
  template <int D>
  struct Drawn {
    float u[D];
    uint32_t hi[(D + 1) / 2];        // high word of each block's odd half
  };
  template <int D>
  __device__ __forceinline__ void peek(Drawn<D>& P, const PhiloxRK& R) const {
    constexpr int NB = (D + 1) / 2;
    const bool odd = (n & 1ull) != 0;
    const uint64_t b0 = (n + 1) >> 1;
    uint32_t h[2 * NB];
#pragma unroll
    for (int k = 0; k < NB; ++k) {
      const uint64_t blk = b0 + (uint64_t)k;
      const uint4 o = philox_rk(make_uint4((uint32_t)blk, (uint32_t)(blk >> 32), k0, k1), R);
      h[2 * k] = o.y;
      h[2 * k + 1] = o.w;
      P.hi[k] = o.w;
    }
    const uint32_t sp = (uint32_t)(spare >> 32);
#pragma unroll
    for (int j = 0; j < D; ++j) {
      const uint32_t w = odd ? (j == 0 ? sp : h[j > 0 ? j - 1 : 0]) : h[j];
      P.u[j] = __uint2float_rn(w >> 8) * 0x1p-24f;
    }
  }
  template <int D>
  __device__ __forceinline__ void advance(const Drawn<D>& P, int used) {
    if (used <= 0) return;
    const uint64_t b0 = (n + 1) >> 1;
    n += (uint64_t)used;
    if (n & 1ull) {
      const uint64_t k = (n >> 1) - b0;
      uint32_t w = 0;
#pragma unroll
      for (int j = 0; j < (D + 1) / 2; ++j)
        if ((uint64_t)j == k) w = P.hi[j];
      spare = (uint64_t)w << 32;
    }
  }
};

// u[i] for a runtime index i known to lie in [LO, HI], by HI - LO selects
// (no indexed, local-memory access)
template <int LO, int HI, int D>
__device__ __forceinline__ float pick_in(const float (&u)[D], int i) {
  static_assert(0 <= LO && LO <= HI && HI < D, "pick_in range");
  float r = u[LO];
#pragma unroll
  for (int j = LO + 1; j <= HI; ++j)
    if (j == i) r = u[j];
  return r;
}

// --------------------------------------------------- non-contracting float64
// The reference evaluates expressions one rounding per operation (numpy
// scalars).  Where a formula is ill-conditioned (1 - beta^2, arccos near 1,
// sqrt(1 - c^2)) a fused multiply-add changes the result far beyond the last
// place, so those code paths use S, whose operators never fuse.
struct S {
  double v;
  __device__ __forceinline__ S() : v(0) {}
  __device__ __forceinline__ S(double x) : v(x) {}
  __device__ __forceinline__ operator double() const { return v; }
};
__device__ __forceinline__ S operator+(S a, S b) { return S(__dadd_rn(a.v, b.v)); }
__device__ __forceinline__ S operator-(S a, S b) { return S(__dsub_rn(a.v, b.v)); }
__device__ __forceinline__ S operator*(S a, S b) { return S(__dmul_rn(a.v, b.v)); }
__device__ __forceinline__ S operator/(S a, S b) { return S(__ddiv_rn(a.v, b.v)); }
__device__ __forceinline__ S operator-(S a) { return S(-a.v); }
__device__ __forceinline__ S sq(S a) { return a * a; }
__device__ __forceinline__ S ssqrt(S a) { return S(__dsqrt_rn(a.v)); }

// numpy.linalg.norm of a 3-vector: sqrt of a sequential fused dot product.
__device__ __forceinline__ double norm3_np(double x, double y, double z) {
  return __dsqrt_rn(__fma_rn(z, z, __fma_rn(y, y, __dmul_rn(x, x))));
}

// ------------------------------------------------------------ warp helpers
__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Each lane of the currently converged group asks for `want` in {0,1,2}
// slots of `counter`; one atomic per group.  Returns this lane's first slot.
__device__ __forceinline__ unsigned long long warp_reserve(unsigned long long* counter, int want) {
  const unsigned mask = __activemask();
  const unsigned b1 = __ballot_sync(mask, want >= 1);
  const unsigned b2 = __ballot_sync(mask, want >= 2);
  const unsigned lt = lanemask_lt();
  const unsigned prefix = __popc(b1 & lt) + __popc(b2 & lt);
  const unsigned total = __popc(b1) + __popc(b2);
  const int leader = __ffs(mask) - 1;
  unsigned long long base = 0;
  if ((int)(threadIdx.x & 31) == leader && total) base = atomicAdd(counter, (unsigned long long)total);
  base = __shfl_sync(mask, base, leader);
  return base + prefix;
}

}  // namespace pt
