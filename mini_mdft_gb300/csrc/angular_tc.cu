// angular_tc.cu -- orientation <-> projection transforms on the tensor cores.
//
// At one grid point both transforms are fixed linear maps (host_setup.cpp:
// ang_matrix_a2p, (2 np) x no, and ang_matrix_p2a, no x (2 np): the rfft2 over
// (phi, psi), the conjugation, the theta contraction with the Wigner-d,
// quadrature and sqrt(2m+1) factors of
// common/MDFT_OrientationProjectionTransform.hpp:270-380, and the synthesis
// and C2R transform of :391-484, folded into one dense matrix).  Over all
// grid points each transform is therefore one GEMM,
//     out[point, j] = sum_k in[point, k] T[j, k],
// with M = grid points (128 per tile), N = outputs per point, K = inputs per
// point; it runs on the fifth-generation tensor cores (tcgen05.mma, operands
// in shared memory, FP32 accumulators in tensor memory).
//
// Precision: the products must be as accurate as the form's arithmetic
// (FP64 fields: about 2^-48; FP32: about 2^-24), which BF16 inputs cannot
// give directly.  Both operands are cut into exact digit slices (error-free
// transformation of matrix products, Ozaki, Ogita, Oishi and Rump 2012).  With a
// power-of-two scale 2^E per row (grid point) of the input and 2^F per output
// column of the matrix, each value scaled to a 7 SL-bit integer is cut into
// SL balanced base-128 digits (top digit in [-128, 128], the others in
// [-64, 63]),
//     x = 2^E sum_s d_s 128^-s,   T = 2^F sum_t e_t 128^-t,
// every digit exact in BF16.  The top digits' product is at most 2^14 and
// any other digit product at most 2^13, and a level adds at most
// min(LMAX - 1, SL) of them per k, so while those bounds times K stay below
// 2^24 each MMA level
//     acc_L = sum_{s + t = L} sum_k d_s(k) e_t(k),  L = 2..LMAX
// is an exact integer in its FP32 accumulator, and
//     out = 2^(E + F) sum_L acc_L 128^-L
// is formed in the epilogue.  FP64 fields: SL = 7 (49 bits), LMAX = 8 (28
// MMAs per 16-wide K step, K <= 288), the sum formed exactly in integer
// arithmetic and rounded once to double, error near 2^-48 of the row and
// column scales.  FP32 fields: SL = 4 (28 bits), LMAX = 5 (10 MMAs), the
// sum formed in FP32.  Cutting FP32 values into three BF16 pieces whose
// products accumulate as floats (6 MMAs) was measured first: its per-value
// errors were FP32-sized, but the energy of the 32^3 pipeline test moved by
// 1.3e-6 (bound 1e-6) -- the tensor core's FP32 accumulation does not round
// like FP32 arithmetic -- while exact digits keep every level sum exact.
//
// Persistent CTAs (one per SM, 512 threads) walk over tiles of 128 grid
// points.  A tile's inputs arrive in shared memory by bulk asynchronous
// copies (one contiguous run of point-major orientation values, or one run of
// 128 complex values per projection plane); the next tile's copy is issued as
// soon as the current tile's last chunk is cut, so it lands under the last
// MMAs and the epilogue.  For digit slicing, the row exponent of each point
// comes from a pass over its staged inputs.  Then, per 16-wide K chunk, the
// threads cut the chunk into slices in shared memory (canonical K-major
// layout without swizzling: 8-row x 16-byte core matrices), and one thread
// issues the MMAs against the matrix's slices (copied into shared memory once
// per CTA) into tensor memory and commits them to an mbarrier; the chunk
// stages are double-buffered, so cutting chunk c+1 overlaps the MMAs of chunk
// c.  After the last chunk each warp reads its 32 tensor-memory lanes (its
// points) and writes the outputs: p in (np, N) layout (consecutive threads,
// consecutive points) or o in point-major layout.
#include <algorithm>
#include <cmath>

#include "tc.cuh"

namespace mdft {

namespace {

constexpr int kTcRows = 128;     // grid points per tile (MMA M)
constexpr int kTcMaxCols = 512;  // padded outputs per point (nnc NC)

// Digits per operand (SL), highest level (LMAX: levels 2..LMAX, one
// accumulator each) and N-chunk width limit of each form.
template <typename S>
struct TcForm;
template <>
struct TcForm<double> {
  static constexpr int SL = 7, LMAX = 8, NACC = LMAX - 1, NCMAX = 64;
};
template <>
struct TcForm<float> {
  static constexpr int SL = 4, LMAX = 5, NACC = LMAX - 1, NCMAX = 128;
};

// ---- exponent and digits of one input value ----------------------------------
// Biased exponent field (0 for zero and subnormals, which become zero digits).
__device__ __forceinline__ int exp_field(double x) {
  return (int)((unsigned long long)__double_as_longlong(x) >> 52) & 0x7ff;
}
__device__ __forceinline__ int exp_field(float x) { return (int)(__float_as_uint(x) >> 23) & 0xff; }
// Row scale exponent E from the largest exponent field: |x| < 2^E.
__device__ __forceinline__ int row_exp(int emax, double) { return emax - 1022; }
__device__ __forceinline__ int row_exp(int emax, float) { return emax - 126; }

// Small integers as floats without the conversion pipe: a 7-bit field u
// becomes 2^23 + u in the mantissa of a float, minus 2^23 + 64 (the balanced
// digit u - 64); v in (-2^22, 2^22): 1.5 2^23 + v, minus 1.5 2^23.
__device__ __forceinline__ float bal2f(unsigned u) { return __uint_as_float(0x4B000000u | u) - 8388672.f; }
__device__ __forceinline__ float i2f(int v) { return __int_as_float(0x4B400000 + v) - 12582912.f; }

// X = round(x 2^(7 SL - E)) cut into SL balanced base-128 digits, most
// significant first: X + 64 (1 + 128 + ... + 128^(SL-2)) holds the lower
// digits plus 64 in its 7-bit fields, and its top bits are the top digit
// (in [-128, 128]); the others lie in [-64, 63].  As floats (small integers,
// exact in BF16).
__device__ __forceinline__ void digits(double x, int E, float (&d)[7]) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int eb = (int)(b >> 52) & 0x7ff;
  long long X = 0;
  if (eb != 0) {
    const unsigned long long m = (b & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    int sh = 1026 + E - eb;  // >= 4 when |x| < 2^E
    sh = sh < 1 ? 1 : sh;
    if (sh < 56) X = (long long)((m + (1ull << (sh - 1))) >> sh);
    if (b >> 63) X = -X;
  }
  constexpr long long kOff = 64LL * (1 + (1LL << 7) + (1LL << 14) + (1LL << 21) + (1LL << 28) + (1LL << 35));
  X += kOff;
  const unsigned lo = (unsigned)X, hi = (unsigned)((unsigned long long)X >> 32);
  d[6] = bal2f(lo & 127u);
  d[5] = bal2f((lo >> 7) & 127u);
  d[4] = bal2f((lo >> 14) & 127u);
  d[3] = bal2f((lo >> 21) & 127u);
  d[2] = bal2f(__funnelshift_r(lo, hi, 28) & 127u);
  d[1] = bal2f((hi >> 3) & 127u);
  d[0] = i2f((int)hi >> 10);
}
// FP32 values: the same digits by exact float arithmetic.  t = x 2^(7 - E)
// (|t| < 128, exact); each step takes the nearest integer d of t (by the
// 1.5 2^23 rounding trick, |t| < 2^22), keeps t - d (exact, |t - d| <= 1/2)
// and scales it by 128 (exact).  The digits come out balanced (|d| <= 64
// after the first) and the last one is rounded, as round(x 2^(28 - E)) is.
__device__ __forceinline__ void digits(float x, int E, float (&d)[4]) {
  float t = x * __int_as_float((134 - E) << 23);  // 2^(7 - E), E in [-126, 129]
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    const float r = (t + 12582912.f) - 12582912.f;
    d[s] = r;
    t = (t - r) * 128.f;
  }
}
// two BF16 values (the high halves of two floats that are exact in BF16)
// packed low-first
__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  return __byte_perm(__float_as_uint(lo), __float_as_uint(hi), 0x7632);
}

// ---- epilogue: sum_L acc_L 128^-L scaled by 2^e -------------------------------
// FP64 fields: the levels are exact integers; V = sum_L acc_L 128^(LMAX-L) / 8
// is formed in 64-bit integer arithmetic (|V| < 2^62 for K <= 288; the
// lowest level loses its three low bits, 2^-52 of the scale) and rounded
// once to the nearest double; then the exponent is adjusted.
template <int LMAX>
__device__ __forceinline__ double combine(const float* acc, int e) {
  long long V = 0;
#pragma unroll
  for (int L = 2; L <= LMAX; ++L) {
    const long long a = (long long)__float2int_rn(acc[L - 2]);
    const int sh = 7 * (LMAX - L) - 3;
    V += sh >= 0 ? a * (1LL << sh) : (a >> (-sh));
  }
  if (V == 0) return 0.0;
  const unsigned long long sgn = V < 0 ? (1ull << 63) : 0ull;
  const unsigned long long u = V < 0 ? (unsigned long long)(-V) : (unsigned long long)V;
  const int top = 63 - __clzll((long long)u);  // leading bit position
  long long ex = top;
  unsigned long long mant;
  if (top > 52) {
    const int sh = top - 52;
    const unsigned long long half = 1ull << (sh - 1);
    const unsigned long long rem = u & ((1ull << sh) - 1);
    mant = u >> sh;
    if (rem > half || (rem == half && (mant & 1ull))) ++mant;
    if (mant >> 53) {  // rounding carried into a new bit
      mant >>= 1;
      ++ex;
    }
  } else {
    mant = u << (52 - top);
  }
  // 2^(e + 3 - 7 LMAX) scale folded into the exponent
  const long long be = ex + 1023 + e + 3 - 7 * LMAX;
  if (be <= 0) return sgn ? -0.0 : 0.0;  // below the normal range of the fields
  if (be >= 2047) return __longlong_as_double((long long)(sgn | 0x7FF0000000000000ull));
  return __longlong_as_double((long long)(sgn | ((unsigned long long)be << 52) | (mant & 0xFFFFFFFFFFFFFull)));
}
// FP32 fields: the levels summed in FP32 from the smallest (Horner in 2^-7),
// then scaled by 2^(e - 14)
__device__ __forceinline__ float pow2f(int e) { return __int_as_float((e + 127) << 23); }
template <int LMAX>
__device__ __forceinline__ float combine_f(const float* acc, int e) {
  float v = acc[LMAX - 2];
#pragma unroll
  for (int L = LMAX - 1; L >= 2; --L) v = fmaf(v, 0.0078125f, acc[L - 2]);
  return v * pow2f(e - 14);
}

// Roles: warps 0..15 produce (row exponents, digit slices, epilogue), warp 16
// allocates the tensor memory and its lane 0 issues the copies and the MMAs.
// They meet only on mbarriers: full[st] (16 producer-warp arrivals: stage st
// cut), empty[st] (MMA commit: stage st read), acc_full (MMA commit: an
// N-pass's accumulators final), acc_empty (16 arrivals: the epilogue has read
// them), raw_full (bulk copy of a tile landed), raw_empty (16 arrivals: the
// tile's last chunk is cut), mat (the matrix landed).  Every wait is bounded;
// a wait that runs out raises `abort` in shared memory, which every other
// wait also watches, so all roles leave their loops and meet at the end.
constexpr int kProducers = 512;
constexpr int kTcCta = kProducers + 32;

template <typename S, int DIR>
__global__ void __launch_bounds__(kTcCta, 1)
ang_tc_kernel(const AngTcDir D, long long N, long long pstride, int bulk_ok, const S* __restrict__ in,
              S* __restrict__ out, int* __restrict__ err, int* __restrict__ flag) {
  using F = TcForm<S>;
  constexpr int SL = F::SL, NACC = F::NACC;
  constexpr uint32_t A_SLICE = kTcRows * 16 * 2;  // 128 rows x 16 k x BF16
  extern __shared__ __align__(128) unsigned char sm[];
  // 0 raw_full, 1 raw_empty, 2/3 full, 4/5 empty, 6 acc_full, 7 acc_empty, 8 mat
  __shared__ __align__(8) unsigned long long bars[9];
  __shared__ uint32_t holder;
  __shared__ volatile int abort_flag;
  __shared__ int rowE[kTcRows];
  __shared__ int epart[4][kTcRows];
  __shared__ int fexp_s[kTcMaxCols];

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int NC = D.NC, K = D.K;
  const uint32_t B_SLICE = (uint32_t)NC * 32;
  S* raw = reinterpret_cast<S*>(sm);
  unsigned char* Abuf = sm + D.raw_bytes;
  unsigned char* Bbuf = Abuf + 2 * SL * A_SLICE;  // the whole matrix, every chunk (resident)
  const long long ntiles = (N + kTcRows - 1) / kTcRows;
  const int np = K / 2;  // projections (proj2angl input)
  auto bar = [&](int i) { return tc::smem_addr(&bars[i]); };
  auto tile_cnt = [&](long long t) { return (int)min((long long)kTcRows, N - t * kTcRows); };
  auto tile_bulk = [&](long long t) { return bulk_ok && tile_cnt(t) == kTcRows; };
  // bounded wait that also gives up once another role has aborted
  auto wait = [&](int i, uint32_t parity) {
    for (int rep = 0; rep < 64; ++rep) {
      if (abort_flag) return false;
      if (tc::mbar_wait(bar(i), parity, tc::kWaitLimit / 64)) return true;
    }
    abort_flag = 1;
    return false;
  };
  auto arrive = [&](int i) { asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar(i)) : "memory"); };
  auto psync = [&] { asm volatile("bar.sync 1, %0;" ::"n"(kProducers) : "memory"); };  // producers only

  if (tid == 0) {
    for (int i = 0; i < 9; ++i) tc::mbar_init(bar(i), (i == 1 || i == 2 || i == 3 || i == 7) ? kProducers / 32 : 1);
    tc::mbar_fence_init();
    abort_flag = 0;
  }
  for (int j = tid; j < D.nnc * NC; j += kTcCta) fexp_s[j] = D.fexp[j];
  if (warp == kProducers / 32) tc::tmem_alloc(tc::smem_addr(&holder), (uint32_t)D.tcols);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tbase = holder;
  const int npass = D.nnc;

  if (warp == kProducers / 32) {
    // ================= MMA warp: lane 0 issues copies and MMAs =================
    if (lane == 0) {
      const uint32_t raw_addr = tc::smem_addr(raw);
      auto issue_raw = [&](long long t) {
        const long long pt0 = t * kTcRows;
        if (DIR == 0) {
          const uint32_t bytes = (uint32_t)(kTcRows * K * sizeof(S));
          tc::mbar_expect_tx(bar(0), bytes);
          tc::bulk_g2s(raw_addr, in + pt0 * K, bytes, bar(0));
        } else {
          const uint32_t bytes = (uint32_t)(kTcRows * 2 * sizeof(S));
          tc::mbar_expect_tx(bar(0), bytes * np);
          for (int ip = 0; ip < np; ++ip)
            tc::bulk_g2s(raw_addr + ip * bytes, in + ((long long)ip * pstride + pt0) * 2, bytes, bar(0));
        }
      };
      const uint32_t mbytes = (uint32_t)D.nnc * D.nkc * SL * B_SLICE;
      tc::mbar_expect_tx(bar(8), mbytes);
      tc::bulk_g2s(tc::smem_addr(Bbuf), D.bsl, mbytes, bar(8));
      long long tile = blockIdx.x;
      if (tile < ntiles && tile_bulk(tile)) issue_raw(tile);
      bool ok = wait(8, 0);
      const uint32_t idesc = tc::idesc_bf16_f32(kTcRows, NC);
      // descriptors of stage 0 / slice 0 and of chunk 0 / slice 0; the
      // start-address field (bits 0-13, 16-byte units) takes the offsets
      const uint64_t ad0 = tc::smem_desc(tc::smem_addr(Abuf), 2048, 128);
      const uint64_t bd0 = tc::smem_desc(tc::smem_addr(Bbuf), (uint32_t)NC * 16, 128);
      long long c = 0, pass = 0;
      for (int it = 0; tile < ntiles; tile += gridDim.x, ++it) {
        for (int nc = 0; nc < npass; ++nc, ++pass) {
          if (pass > 0 && ok) ok = wait(7, (uint32_t)((pass - 1) & 1));  // the epilogue has read the accumulators
          for (int kc = 0; kc < D.nkc; ++kc, ++c) {
            const int st = (int)(c & 1);
            if (ok) ok = wait(2 + st, (uint32_t)((c >> 1) & 1));  // stage st cut
            if (ok) {
              tc::fence_after_sync();
              const uint64_t ad = ad0 + ((uint64_t)(st * SL * A_SLICE) >> 4);
              const uint64_t bd = bd0 + ((uint64_t)((nc * D.nkc + kc) * SL * B_SLICE) >> 4);
#pragma unroll
              for (int L = 2; L <= F::LMAX; ++L) {
                const int s0 = max(1, L - SL), s1 = min(SL, L - 1);
                for (int s = s0; s <= s1; ++s)
                  tc::mma_bf16(tbase + (uint32_t)((L - 2) * NC), ad + ((uint64_t)((s - 1) * A_SLICE) >> 4),
                               bd + ((uint64_t)((L - s - 1) * B_SLICE) >> 4), idesc,
                               (kc > 0 || s > s0) ? 1u : 0u);
              }
              tc::mma_commit(bar(4 + st));  // stage st read
            }
            if (nc == npass - 1 && kc == D.nkc - 1) {
              // the next tile's inputs once the producers have cut this tile's last chunk
              const long long nt = tile + gridDim.x;
              if (ok && nt < ntiles && tile_bulk(nt)) {
                ok = wait(1, (uint32_t)(it & 1));
                if (ok) issue_raw(nt);
              }
            }
          }
          if (ok) tc::mma_commit(bar(6));  // accumulators of this pass final
        }
      }
    }
    __syncwarp();
  } else {
    // ================= producers: warps 0..15 =================
    long long c = 0, pass = 0;
    uint32_t ph_raw = 0;
    bool ok = true;
    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
      const long long pt0 = tile * kTcRows;
      const int cnt = tile_cnt(tile);
      // ---- the raw tile in shared memory ----
      if (tile_bulk(tile)) {
        if (ok) ok = wait(0, ph_raw);
        ph_raw ^= 1u;
      } else if (ok) {
        for (int i = tid; i < kTcRows * K; i += kProducers) {
          S v = S(0);
          if (DIR == 0) {
            if (i < cnt * K) v = in[pt0 * K + i];
          } else {
            const int ip = i / (2 * kTcRows), r = (i >> 1) & (kTcRows - 1);
            if (r < cnt) v = in[((long long)ip * pstride + pt0 + r) * 2 + (i & 1)];
          }
          raw[i] = v;
        }
      }
      ok = __all_sync(0xffffffffu, ok);
      psync();
      // ---- row exponents (largest exponent field of each point's inputs) ----
      if (DIR == 0) {  // warp per row, lanes along the contiguous row
        for (int r = warp; r < kTcRows; r += kProducers / 32) {
          int em = 0;
          for (int k = lane; k < K; k += 32) em = max(em, exp_field(raw[r * K + k]));
          em = __reduce_max_sync(0xffffffffu, em);
          if (lane == 0) rowE[r] = row_exp(em, S(0));
        }
      } else {  // thread per (row, quarter of the planes)
        const int r = tid & (kTcRows - 1), qt = tid >> 7;
        int em = 0;
        for (int ip = qt; ip < np; ip += 4)
          em = max(em, max(exp_field(raw[(ip * kTcRows + r) * 2]), exp_field(raw[(ip * kTcRows + r) * 2 + 1])));
        epart[qt][r] = em;
        psync();
        if (tid < kTcRows)
          rowE[tid] = row_exp(max(max(epart[0][tid], epart[1][tid]), max(epart[2][tid], epart[3][tid])), S(0));
      }
      psync();
      for (int nc = 0; nc < npass; ++nc, ++pass) {
        for (int kc = 0; kc < D.nkc; ++kc, ++c) {
          const int st = (int)(c & 1);
          if (c >= 2 && ok) ok = wait(4 + st, (uint32_t)(((c >> 1) - 1) & 1));  // MMAs of chunk c - 2 done
          ok = __all_sync(0xffffffffu, ok);
          if (ok) {
            // cut the A chunk: 4 threads per row, 4 of the 16 columns each
            int r, qk;
            if (DIR == 0) {  // consecutive threads along a row (contiguous raw rows)
              r = tid >> 2;
              qk = tid & 3;
            } else {  // consecutive threads on consecutive points (raw planes)
              r = tid & (kTcRows - 1);
              qk = tid >> 7;
            }
            const int E = rowE[r], kb = kc * 16 + qk * 4;
            float dg[4][SL];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
              const int k = kb + i;
              S v = S(0);
              if (k < K) v = DIR == 0 ? raw[r * K + k] : raw[((k >> 1) * kTcRows + r) * 2 + (k & 1)];
              digits(v, E, dg[i]);
            }
            unsigned char* base =
                Abuf + (size_t)st * SL * A_SLICE + (qk >> 1) * 2048 + (r >> 3) * 128 + (r & 7) * 16 + (qk & 1) * 8;
#pragma unroll
            for (int s = 0; s < SL; ++s) {
              uint2 v;
              v.x = pack_bf16(dg[0][s], dg[1][s]);
              v.y = pack_bf16(dg[2][s], dg[3][s]);
              *reinterpret_cast<uint2*>(base + (size_t)s * A_SLICE) = v;
            }
            tc::fence_proxy_async();
          }
          __syncwarp();
          if (lane == 0) {
            arrive(2 + st);  // this warp's part of stage st is cut
            if (nc == npass - 1 && kc == D.nkc - 1) arrive(1);  // the raw tile is no longer read
          }
        }
        // ---- epilogue: warp (lane quadrant q, column quarter g) ----
        if (ok) ok = wait(6, (uint32_t)(pass & 1));
        ok = __all_sync(0xffffffffu, ok);
        if (ok) {
          tc::fence_after_sync();
          const int q = warp & 3, g = warp >> 2, r = q * 32 + lane;
          const int E = rowE[r];
          const int cw = NC / 4;
          for (int c4 = 0; c4 < cw; c4 += 4) {
            const int col = g * cw + c4;
            float a[NACC][4];
#pragma unroll
            for (int L = 0; L < NACC; ++L)
              tc::tmem_ld4(tbase + ((uint32_t)(q * 32) << 16) + (uint32_t)(L * NC + col), a[L]);
            tc::tmem_wait_ld();
            const int j0 = nc * NC + col;
            if (r < cnt) {
#pragma unroll
              for (int i = 0; i < 4; i += 2) {
                const int j = j0 + i;
                if (j >= D.NOUT) break;
                float l0[NACC], l1[NACC];
#pragma unroll
                for (int L = 0; L < NACC; ++L) {
                  l0[L] = a[L][i];
                  l1[L] = a[L][i + 1];
                }
                S v0, v1;
                if constexpr (sizeof(S) == 8) {
                  v0 = combine<F::LMAX>(l0, E + fexp_s[j]);
                  v1 = combine<F::LMAX>(l1, E + fexp_s[j + 1]);
                } else {
                  v0 = combine_f<F::LMAX>(l0, E + fexp_s[j]);
                  v1 = combine_f<F::LMAX>(l1, E + fexp_s[j + 1]);
                }
                if (DIR == 0) {  // columns 2 ip, 2 ip + 1 -> p(ip, point)
                  Cx<S> z;
                  z.re = v0;
                  z.im = v1;
                  reinterpret_cast<Cx<S>*>(out)[(long long)(j >> 1) * pstride + pt0 + r] = z;
                } else {
                  S* o = out + (pt0 + r) * (long long)D.NOUT + j;
                  o[0] = v0;
                  if (j + 1 < D.NOUT) o[1] = v1;
                }
              }
            }
          }
          tc::fence_before_sync();
        }
        __syncwarp();
        if (lane == 0) arrive(7);  // this warp has read the accumulators
      }
      psync();  // rowE and raw are free for the next tile
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (tid == 0 && abort_flag) {
    note_wait_timeout(err, flag);
    // copies or MMAs may still run: wait once more (bounded) before the
    // tensor memory they write is freed
    for (int i = 0; i < 9; ++i) tc::mbar_wait(bar(i), 0, tc::kWaitLimit / 16);
  }
  __syncthreads();
  tc::fence_after_sync();
  if (warp == kProducers / 32) tc::tmem_dealloc(tbase, (uint32_t)D.tcols);
}

// host: the digits of round(x 2^(7 SL - F)) by the same rule as digits() on
// the device (balanced base-128 digits through the offset of 64 per lower
// digit)
template <int SL>
void host_digits(double x, int F, int* d) {
  long long X = std::llround(std::ldexp(x, 7 * SL - F));
  for (int s = 0; s < SL - 1; ++s) X += 64LL << (7 * s);
  for (int s = SL - 1; s >= 1; --s) d[s] = (int)(((unsigned long long)X >> (7 * (SL - 1 - s))) & 127u) - 64;
  d[0] = (int)(X >> (7 * (SL - 1)));
}

uint16_t bf16_bits_of_int(int v) {
  const float f = (float)v;  // |v| <= 128: exact, low 16 bits zero
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return (uint16_t)(u >> 16);
}

}  // namespace

template <typename S>
bool ang_tc_setup(AngTcDir& D, const std::vector<double>& T, int nout, int k, int dir, DevBuf& bsl,
                  DevBuf& fexp) {
  using Fm = TcForm<S>;
  constexpr int SL = Fm::SL, LMAX = Fm::LMAX;
  D.K = k;
  D.nkc = (k + 15) / 16;
  D.NOUT = nout;
  D.nnc = (nout + Fm::NCMAX - 1) / Fm::NCMAX;
  D.NC = ((nout + D.nnc - 1) / D.nnc + 15) / 16 * 16;
  const int ncols = Fm::NACC * D.NC;
  int tc = 32;
  while (tc < ncols) tc *= 2;
  D.tcols = tc;
  // exact sums: the top digits' product is at most 2^14, every other digit
  // product at most 2^13, and level L >= 3 adds at most min(L - 1, SL) of
  // them per k, so every level's K-sum stays below 2^24 while
  // K 2^14 < 2^24 and (pairs) K 2^13 < 2^24
  const int pairs = std::min(LMAX - 1, SL);
  const long long kp = (long long)D.nkc * 16;
  if (kp * 16384 >= (1LL << 24) || pairs * kp * 8192 >= (1LL << 24)) return false;
  if (tc > 512 || (k & 1) || D.nnc * D.NC > kTcMaxCols) return false;
  // shared memory: the raw tile, A (2 stages x SL slices x 4 KB) and the
  // whole matrix B (every chunk: nnc nkc SL NC 32 bytes)
  D.raw_bytes = ((size_t)kTcRows * k * sizeof(S) + 127) & ~size_t(127);
  D.smem = D.raw_bytes + (size_t)2 * SL * kTcRows * 32 + (size_t)D.nnc * D.nkc * SL * D.NC * 32;
  int dev = 0, optin = 0;
  cuda_check(cudaGetDevice(&dev), "cudaGetDevice");
  cuda_check(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev), "smem opt-in");
  cudaFuncAttributes fa;
  cuda_check(dir == 0 ? cudaFuncGetAttributes(&fa, ang_tc_kernel<S, 0>) : cudaFuncGetAttributes(&fa, ang_tc_kernel<S, 1>),
             "angular tensor-core kernel attributes");
  if (D.smem + fa.sharedSizeBytes > (size_t)optin) return false;  // static shared memory counts too
  cuda_check(cudaDeviceGetAttribute(&D.nsm, cudaDevAttrMultiProcessorCount, dev), "SM count");
  // column exponents: |T[j, k]| < 2^F_j over the row
  const int ncp = D.nnc * D.NC;
  std::vector<int> F((size_t)ncp, -1022);
  for (int j = 0; j < nout; ++j) {
    double m = 0;
    for (int kk = 0; kk < k; ++kk) m = std::max(m, std::fabs(T[(size_t)j * k + kk]));
    if (m > 0) {
      int e;
      std::frexp(m, &e);  // m = f 2^e, 0.5 <= f < 1: m < 2^e
      F[j] = e;
    }
  }
  // digit slices in the shared-memory layout of one chunk:
  // (nnc, nkc, SL, kg 2, ng NC/8, row 8, k 8), BF16 bits
  std::vector<uint16_t> B((size_t)D.nnc * D.nkc * SL * D.NC * 16, 0);
  uint16_t sl[SL];
  for (int j = 0; j < nout; ++j)
    for (int kk = 0; kk < k; ++kk) {
      const double t = T[(size_t)j * k + kk];
      int dg[SL];
      host_digits<SL>(t, F[j], dg);
      for (int s = 0; s < SL; ++s) sl[s] = bf16_bits_of_int(dg[s]);
      const int nc = j / D.NC, jn = j % D.NC, kc = kk / 16, kin = kk % 16;
      for (int s = 0; s < SL; ++s) {
        const size_t off = ((((size_t)(nc * D.nkc + kc) * SL + s) * 2 + kin / 8) * (D.NC / 8) + jn / 8) * 64 +
                           (jn % 8) * 8 + kin % 8;
        B[off] = sl[s];
      }
    }
  bsl.upload(B.data(), sizeof(uint16_t) * B.size());
  fexp.upload(F.data(), sizeof(int) * F.size());
  D.bsl = bsl.as<uint16_t>();
  D.fexp = fexp.as<int>();
  if (dir == 0)
    allow_max_smem(ang_tc_kernel<S, 0>, D.smem, "angular tensor-core smem attribute");
  else
    allow_max_smem(ang_tc_kernel<S, 1>, D.smem, "angular tensor-core smem attribute");
  return true;
}

template <typename S>
void ang_tc_launch(const AngPlan& P, int dir, const S* in, S* out, cudaStream_t s) {
  if (P.N == 0) return;
  const AngTcDir& D = dir == 0 ? P.tc_a2p : P.tc_p2a;
  const long long ntiles = (P.N + kTcRows - 1) / kTcRows;
  const long long nb = std::min<long long>(ntiles, D.nsm);
  // whole tiles move by bulk copies when every source address is 16-byte
  // aligned: the base pointer, the row stride (angl2proj: K values per
  // point) or the plane stride (proj2angl: N complex values per projection)
  const uintptr_t base = reinterpret_cast<uintptr_t>(in);
  const bool bulk_ok = (base % 16 == 0) && (dir == 0 ? (D.K * sizeof(S)) % 16 == 0
                                                      : (P.N * 2 * sizeof(S)) % 16 == 0);
  const WaitStatus& w = device_wait_status();
  clear_stale_error();
  if (dir == 0)
    ang_tc_kernel<S, 0><<<(unsigned)nb, kTcCta, D.smem, s>>>(D, P.N, P.N, bulk_ok ? 1 : 0, in, out, w.count,
                                                                   w.flag_dev);
  else
    ang_tc_kernel<S, 1><<<(unsigned)nb, kTcCta, D.smem, s>>>(D, P.N, P.N, bulk_ok ? 1 : 0, in, out, w.count,
                                                                   w.flag_dev);
  launch_check("angular tensor-core kernel launch");
}

template bool ang_tc_setup<double>(AngTcDir&, const std::vector<double>&, int, int, int, DevBuf&, DevBuf&);
template bool ang_tc_setup<float>(AngTcDir&, const std::vector<double>&, int, int, int, DevBuf&, DevBuf&);
template void ang_tc_launch<double>(const AngPlan&, int, const double*, double*, cudaStream_t);
template void ang_tc_launch<float>(const AngPlan&, int, const float*, float*, cudaStream_t);

}  // namespace mdft
