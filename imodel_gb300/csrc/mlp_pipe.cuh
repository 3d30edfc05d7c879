// Pipelined forward pass of the per-edge MLP (internal header of mlp.cu).
//
// One persistent CTA per SM, warp-specialised:
//   NG groups     gather groups (warps 0 .. 4 NG - 1): each turns the index block of
//                 one tile of 128 rows into the tile's BF16 input operand
//                 (the dependent gathers of velocities etc.) and one FP32
//                 context value per row
//   6 - NG groups epilogue groups: TMEM -> registers, GELU, the
//                 BF16 hidden layer back to shared memory, and after the
//                 second product the final GELU . w3 + b3 and the output
//                 (2 GELU is formed, with W2 and w3 halved: exact)
//   warp  24      one thread runs an event loop that issues the bulk copies
//                 (TMA, cp.async.bulk) of each tile's index block and the
//                 tcgen05 MMAs of both layers
// Shared memory holds NPF prefetched index blocks, NSTAGE input operands
// (8 KiB each), NSLOT hidden-layer operands (20 KiB each); TMEM holds NSLOT
// tiles in flight, SLOTW = 80 columns each.  The first product has N = 80:
// columns 0..63 are the hidden units and column 64 carries the row's context
// value through the tensor core (the gather writes it as a BF16 pair hi + lo
// into the zero-padded input columns 24 and 25, and output row 64 of the
// layer-1 operand holds ones there), so it needs no ring buffer of its own;
// the second product overwrites columns 0..63 once the first epilogue has
// read them.  Every hand-off is an mbarrier; every wait is bounded and gives
// up once any role has raised the CTA's abort flag, so a stuck pipeline ends
// with an error flag, never a hang.
//
// Tile i of this CTA (global tile blockIdx.x + i * gridDim.x) uses
//   index block  i % NPF,   input stage  i % NSTAGE  (gather group i % NG),
//   TMEM slot    i % NSLOT  (epilogue group i % NE).
// Phase parities: the j-th completion of a barrier is awaited with parity
// j & 1; a producer waiting for the consumer's (j-1)-th release waits with
// parity (j & 1) ^ 1, which a fresh barrier satisfies at once for j = 0.
#pragma once

namespace imodel {
namespace pipe {

using namespace tc05;

// NGROUPS warp groups of 4 warps are split between gathering (NG) and the
// epilogue (NGROUPS - NG); the split is a tuning choice (2, 3 or 4 gather
// groups), the thread count and register budget are the same for all.
constexpr int NGROUPS = 6, NSTAGE = 4, NSLOT = 6, NPF = 4;
constexpr int N1 = 80, SLOTW = 80;  // layer-1 outputs: 64 hidden units, context, padding
constexpr int K2 = 80;               // layer-2 inputs: 64 hidden units, two ones, padding
constexpr int A2_BYTES = TM * K2 * 2;
constexpr int WARPS = NGROUPS * 4 + 1;
constexpr int THREADS = WARPS * 32;
constexpr int PF_BYTES = 11264;  // largest index block of a task
// dynamic shared memory: B1 5K | B2 10K | A1 ring 32K | A2 slots 120K |
// index blocks 44K
constexpr int OFF_B1S = 0, OFF_B2S = N1 * K1 * 2, OFF_A1S = OFF_B2S + NH * K2 * 2,
              OFF_A2S = OFF_A1S + NSTAGE * 8192, OFF_PF = OFF_A2S + NSLOT * A2_BYTES,
              SMEM = OFF_PF + NPF * PF_BYTES;
static_assert(NSLOT * SLOTW <= 512, "TMEM has 512 columns");
static_assert(SMEM > 116 * 1024, "more than half of an SM's shared memory: one CTA per SM");
static_assert(SMEM <= 220 * 1024, "fits the 227 KiB an SM offers one CTA");
constexpr int ERR_PIPE = 16;

struct Bars {
  uint64_t pf_full[NPF], pf_empty[NPF];
  uint64_t a1_full[NSTAGE], a1_empty[NSTAGE];
  uint64_t acc1[NSLOT], a2_full[NSLOT], acc2[NSLOT], tfree[NSLOT];
  uint64_t done;
};

__device__ __forceinline__ void arrive(uint64_t *mbar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(mbar)) : "memory");
}
// one arrival that also announces `bytes` of bulk-copy data to come
__device__ __forceinline__ void arrive_expect_tx(uint64_t *mbar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(mbar)),
               "r"(bytes)
               : "memory");
}
// bulk (untiled TMA) copy global -> shared; both addresses 16-byte aligned,
// size a multiple of 16; completion counted in bytes on the mbarrier
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes,
                                         uint64_t *mbar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(mbar))
      : "memory");
}

__device__ __forceinline__ bool try_wait(uint64_t *mbar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.b32 %0, 1, 0, p;\n\t}\n"
      : "=r"(done)
      : "r"(smem_u32(mbar)), "r"(parity)
      : "memory");
  return done != 0;
}

// non-blocking test of a phase
__device__ __forceinline__ bool test_wait(uint64_t *mbar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.b32 %0, 1, 0, p;\n\t}\n"
      : "=r"(done)
      : "r"(smem_u32(mbar)), "r"(parity)
      : "memory");
  return done != 0;
}

// bounded wait; false once the CTA aborted (or this wait timed out, which
// raises the abort flag and the error flag)
__device__ __forceinline__ bool wait(uint64_t *mbar, uint32_t parity, volatile int *abort,
                                     int *err) {
  for (int it = 0; it < (1 << 20); ++it) {
    if (try_wait(mbar, parity)) return true;
    if ((it & 15) == 15 && *abort) return false;
  }
  atomicOr(err, ERR_PIPE);
  *abort = 1;
  return false;
}
// every lane waits; the warp goes on only if all lanes saw the phase
__device__ __forceinline__ bool wait_warp(uint64_t *mbar, uint32_t parity, volatile int *abort,
                                          int *err) {
  const bool ok = wait(mbar, parity, abort, err);
  return __all_sync(0xffffffffu, ok) != 0;
}

// 32 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void ld32(uint32_t taddr, float (&v)[32]) {
  float a[16], b[16];
  ld16(taddr, a);
  ld16(taddr + 16, b);
  wait_ld();
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    v[i] = a[i];
    v[16 + i] = b[i];
  }
}

// Task interface (see RowsTask and EdgeTask below):
//   uint32_t pf_bytes(tile)                 bytes of the tile's index block
//   void prefetch(tile, dst, mbar)          issues the block's bulk copies
//   Idx load_idx(pf, r)                     row r's indices, from the block
//   float stage(row, live, idx, c[4])       the row's BF16 inputs -> c, returns
//                                           the context value of the row
//   void write(row, y, ctx)                 consumes the network output
template <class Task, int NG>
__global__ void __launch_bounds__(THREADS, 1)
    k_mlp_pipe(Weights W, int64_t n, Task task, int *err) {
  constexpr int NE = NGROUPS - NG;
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ Bars bar;
  __shared__ uint32_t tslot;
  __shared__ int abort_flag;
  __shared__ __align__(16) float sw3[NH];
  uint8_t *B1s = smem + OFF_B1S, *B2s = smem + OFF_B2S;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  volatile int *abort = &abort_flag;

  // Operands that never change.  Input columns 24, 25 of a row hold its
  // context as a BF16 pair hi + lo and columns 26, 27 hold ones; layer 1's
  // operand B1 [80 outputs][32 inputs] is W1 in rows 0..63 with the bias b1
  // as a pair hi + lo against the ones, and the context row 64 (ones against
  // columns 24, 25).  Layer 2's operand B2 [64][80] is W2 / 2 (it multiplies
  // 2 gelu, see gelu2x2; halving is exact) with the bias b2 as a pair against
  // columns 64, 65 of the hidden-layer operand, which hold ones.  The biases
  // thus enter the products with 16 significant bits.
  for (int i = tid; i < 4096 / 16; i += THREADS)
    reinterpret_cast<uint4 *>(B1s)[i] = reinterpret_cast<const uint4 *>(W.w1img)[i];
  for (int i = 4096 / 16 + tid; i < N1 * K1 * 2 / 16; i += THREADS)
    reinterpret_cast<uint4 *>(B1s)[i] = make_uint4(0, 0, 0, 0);
  const uint16_t *w2 = W.w2img;
  for (int i = tid; i < NH * K2; i += THREADS) {
    const int o = i / K2, k = i % K2;
    float v = 0.0f;
    if (k < NH) {
      v = 0.5f * __bfloat162float(__ushort_as_bfloat16(w2[kmaj_off(o, k, NH) / 2]));
    } else if (k < NH + 2) {
      const float b = W.p[OFF_B2 + o];
      const float hi = __bfloat162float(__float2bfloat16_rn(b));
      v = k == NH ? hi : b - hi;
    }
    *reinterpret_cast<uint16_t *>(B2s + kmaj_off(o, k, K2)) = bf16bits(v);
  }
  for (int i = tid; i < NSLOT * TM; i += THREADS) {  // ones in hidden columns 64, 65
    uint8_t *A2 = smem + OFF_A2S + (i / TM) * A2_BYTES;
    const int r = i % TM;
    *reinterpret_cast<uint4 *>(A2 + kmaj_off(r, NH, K2)) = make_uint4(pack2(1.0f, 1.0f), 0, 0, 0);
    *reinterpret_cast<uint4 *>(A2 + kmaj_off(r, NH + 8, K2)) = make_uint4(0, 0, 0, 0);
  }
  __syncthreads();
  if (tid < NH) {
    const float b = W.p[OFF_B1 + tid];
    const float hi = __bfloat162float(__float2bfloat16_rn(b));
    *reinterpret_cast<uint32_t *>(B1s + kmaj_off(tid, 26, K1)) = pack2(hi, b - hi);
    sw3[tid] = 0.5f * W.p[OFF_W3 + tid];
  }
  if (tid == 0) *reinterpret_cast<uint32_t *>(B1s + kmaj_off(64, 24, K1)) = pack2(1.0f, 1.0f);
  if (tid == 0) {
    abort_flag = 0;
    for (int k = 0; k < NPF; ++k) {
      mbar_init(&bar.pf_full[k], 1);
      mbar_init(&bar.pf_empty[k], 128);
    }
    for (int k = 0; k < NSTAGE; ++k) {
      mbar_init(&bar.a1_full[k], 128);
      mbar_init(&bar.a1_empty[k], 1);
    }
    for (int k = 0; k < NSLOT; ++k) {
      mbar_init(&bar.acc1[k], 1);
      mbar_init(&bar.a2_full[k], 128);
      mbar_init(&bar.acc2[k], 1);
      mbar_init(&bar.tfree[k], 128);
    }
    mbar_init(&bar.done, 1);
  }
  if (warp == 0) tmem_alloc(&tslot, 512);
  fence_async_smem();
  sync_cta();
  const uint32_t tmem = tslot;
  const float b3 = W.p[OFF_B3];
  const int64_t ntiles = (n + TM - 1) / TM;
  const int ntile_cta =
      blockIdx.x < ntiles ? static_cast<int>((ntiles - 1 - blockIdx.x) / gridDim.x + 1) : 0;
  auto tile_of = [&](int i) { return blockIdx.x + static_cast<int64_t>(i) * gridDim.x; };

  if (warp < NG * 4) {
    // ---- gather groups -----------------------------------------------------
    const int g = warp >> 2, r = tid & 127;
    for (int i = g; i < ntile_cta; i += NG) {
      const int p = i % NPF, s = i % NSTAGE;
      if (!wait_warp(&bar.pf_full[p], (i / NPF) & 1, abort, err)) break;
      const auto idx = task.load_idx(smem + OFF_PF + p * PF_BYTES, r);
      arrive(&bar.pf_empty[p]);
      const int64_t row = tile_of(i) * TM + r;
      uint4 c[4];
      const float cx = task.stage(row, row < n, idx, c);
      // the context as hi + lo in input columns 24, 25 (16 significant bits),
      // ones in columns 26, 27 (the bias of layer 1)
      const float hi = __bfloat162float(__float2bfloat16_rn(cx));
      c[3] = make_uint4(pack2(hi, cx - hi), pack2(1.0f, 1.0f), 0, 0);
      if (!wait_warp(&bar.a1_empty[s], ((i / NSTAGE) & 1) ^ 1, abort, err)) break;
      uint8_t *A1 = smem + OFF_A1S + s * 8192;
#pragma unroll
      for (int q = 0; q < 4; ++q) *reinterpret_cast<uint4 *>(A1 + kmaj_off(r, 8 * q, K1)) = c[q];
      fence_async_smem();
      arrive(&bar.a1_full[s]);
    }
  } else if (warp < NGROUPS * 4) {
    // ---- epilogue groups ---------------------------------------------------
    const int e = (warp - NG * 4) >> 2, r = tid & 127;
    const uint32_t lane_base = static_cast<uint32_t>((warp & 3) * 32) << 16;
    for (int i = e; i < ntile_cta; i += NE) {
      const int t = i % NSLOT;
      const uint32_t par = (i / NSLOT) & 1;
      const uint32_t tcol = tmem + lane_base + t * SLOTW;
      if (!wait_warp(&bar.acc1[t], par, abort, err)) break;
      fence_after_sync();
      uint8_t *A2 = smem + OFF_A2S + t * A2_BYTES;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        float v[32];
        ld32(tcol + 32 * h, v);
#pragma unroll
        for (int c8 = 0; c8 < 4; ++c8) {
          const float *w = v + 8 * c8;
          float gv[8];
          f2upk(gelu2x2(w[0], w[1]), gv[0], gv[1]);
          f2upk(gelu2x2(w[2], w[3]), gv[2], gv[3]);
          f2upk(gelu2x2(w[4], w[5]), gv[4], gv[5]);
          f2upk(gelu2x2(w[6], w[7]), gv[6], gv[7]);
          uint4 q;
          q.x = pack2(gv[0], gv[1]);
          q.y = pack2(gv[2], gv[3]);
          q.z = pack2(gv[4], gv[5]);
          q.w = pack2(gv[6], gv[7]);
          *reinterpret_cast<uint4 *>(A2 + kmaj_off(r, 32 * h + 8 * c8, K2)) = q;
        }
      }
      float cv[16];
      ld16(tcol + 64, cv);
      wait_ld();
      const float cx = cv[0];
      fence_async_smem();
      fence_before_sync();
      arrive(&bar.a2_full[t]);
      if (!wait_warp(&bar.acc2[t], par, abort, err)) break;
      fence_after_sync();
      // even and odd hidden units summed in the two lanes of a pair
      uint64_t acc2 = 0;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        float v[32];
        ld32(tcol + 32 * h, v);
#pragma unroll
        for (int c4 = 0; c4 < 8; ++c4) {
          const float4 wq = reinterpret_cast<const float4 *>(sw3)[8 * h + c4];
          const float *w = v + 4 * c4;
          acc2 = f2fma(gelu2x2(w[0], w[1]), f2pk(wq.x, wq.y), acc2);
          acc2 = f2fma(gelu2x2(w[2], w[3]), f2pk(wq.z, wq.w), acc2);
        }
      }
      float acc_e, acc_o;
      f2upk(acc2, acc_e, acc_o);
      const float acc = b3 + (acc_e + acc_o);
      fence_before_sync();
      arrive(&bar.tfree[t]);
      const int64_t row = tile_of(i) * TM + r;
      if (row < n) task.write(row, acc, cx);
    }
  } else if (lane == 0) {
    // ---- producer and MMA issuer (one thread; the warp's other lanes wait
    // below).  An event loop: the index block of tile ip is fetched as soon
    // as its buffer is free; the first layer of tile i1 is issued as soon as
    // its inputs are staged and its TMEM slot is free; the second layer of
    // tile i2 as soon as its hidden layer is in shared memory.  At most NSLOT
    // tiles are in TMEM at once.
    const uint32_t id80 = idesc_bf16(TM, N1), id64 = idesc_bf16(TM, NH);
    int ip = 0, i1 = 0, i2 = 0;
    for (long long idle = 0; i2 < ntile_cta;) {
      bool progress = false;
      if (ip < ntile_cta && test_wait(&bar.pf_empty[ip % NPF], ((ip / NPF) & 1) ^ 1)) {
        uint64_t *mb = &bar.pf_full[ip % NPF];
        const int64_t tile = tile_of(ip);
        arrive_expect_tx(mb, task.pf_bytes(tile, n));
        task.prefetch(tile, n, smem + OFF_PF + (ip % NPF) * PF_BYTES, mb);
        ++ip;
        progress = true;
      }
      if (i1 < ntile_cta && i1 - i2 < NSLOT &&
          test_wait(&bar.a1_full[i1 % NSTAGE], (i1 / NSTAGE) & 1) &&
          test_wait(&bar.tfree[i1 % NSLOT], ((i1 / NSLOT) & 1) ^ 1)) {
        const int s1 = i1 % NSTAGE, t = i1 % NSLOT;
        fence_after_sync();
        const uint32_t a1 = smem_u32(smem + OFF_A1S + s1 * 8192);
        for (int k = 0; k < K1 / 16; ++k)
          mma(tmem + t * SLOTW, smem_desc(a1 + 256 * k, 128, K1 * 16),
              smem_desc(smem_u32(B1s) + 256 * k, 128, K1 * 16), id80, k);
        commit(&bar.a1_empty[s1]);
        commit(&bar.acc1[t]);
        ++i1;
        progress = true;
      }
      if (i2 < i1 && test_wait(&bar.a2_full[i2 % NSLOT], (i2 / NSLOT) & 1)) {
        const int t = i2 % NSLOT;
        fence_after_sync();
        const uint32_t a2 = smem_u32(smem + OFF_A2S + t * A2_BYTES);
        for (int k = 0; k < K2 / 16; ++k)
          mma(tmem + t * SLOTW, smem_desc(a2 + 256 * k, 128, K2 * 16),
              smem_desc(smem_u32(B2s) + 256 * k, 128, K2 * 16), id64, k);
        commit(&bar.acc2[t]);
        ++i2;
        progress = true;
      }
      if (progress) {
        idle = 0;
      } else if ((++idle & 63) == 0 && (*abort || idle > (1ll << 26))) {
        if (!*abort) {
          atomicOr(err, ERR_PIPE);
          *abort = 1;
        }
        break;
      }
    }
    // every issued MMA and copy has completed before the CTA leaves: the
    // MMAs through this commit, the copies through their own barriers
    commit(&bar.done);
    for (int it = 0; it < (1 << 20) && !try_wait(&bar.done, 0); ++it) {
    }
    // (after an abort: the last index block fetched into each buffer)
    for (int j = ip - NPF > i1 ? ip - NPF : i1; j < ip; ++j)
      for (int it = 0; it < (1 << 20) && !try_wait(&bar.pf_full[j % NPF], (j / NPF) & 1); ++it) {
      }
  }
  __syncwarp();
  sync_cta();
  if (warp == 0) tmem_dealloc(tmem, 512);
}

// ---- tasks: where the rows come from and where the outputs go ---------------
// rows of a BF16 input matrix [n][24] (16-byte aligned) -> y[n]
struct RowsTask {
  const uint16_t *x;
  float *y;
  struct Idx {
    uint4 a, b, c;
  };
  __device__ __forceinline__ uint32_t pf_bytes(int64_t tile, int64_t n) const {
    const int64_t rows = n - tile * TM < TM ? n - tile * TM : TM;
    return static_cast<uint32_t>(rows * NIN * 2);
  }
  __device__ __forceinline__ void prefetch(int64_t tile, int64_t n, uint8_t *dst,
                                           uint64_t *mbar) const {
    bulk_g2s(dst, x + tile * TM * NIN, pf_bytes(tile, n), mbar);
  }
  __device__ __forceinline__ Idx load_idx(const uint8_t *pf, int r) const {
    const uint4 *s = reinterpret_cast<const uint4 *>(pf + r * NIN * 2);
    return Idx{s[0], s[1], s[2]};
  }
  __device__ __forceinline__ float stage(int64_t, bool live, const Idx &d, uint4 (&c)[4]) const {
    const uint4 z = make_uint4(0, 0, 0, 0);
    c[0] = live ? d.a : z;
    c[1] = live ? d.b : z;
    c[2] = live ? d.c : z;
    c[3] = z;
    return 0.0f;
  }
  __device__ __forceinline__ void write(int64_t row, float v, float) const { y[row] = v; }
};

// the learned correction of the shallow-water step: inputs from the stencil
// velocities and geometry of edge e; corr[e] = q_e h_e sigma_e clip(y).
// The inputs of a tile are one 11,264-byte block (LearnedLayout in
// swm_layout.h): lst [10][128] | geo [128][16] BF16 | esh [2][128] |
// evs [128][2], fetched with a single bulk copy.
struct EdgeTask {
  const uint8_t *blocks;  // [ntiles][PF_BYTES]
  const float *u, *q_tr, *hd;
  float h_ref;
  float *corr;
  static constexpr int B_LST = 0, B_GEO = 5120, B_ESH = 9216, B_EVS = 10240;
  struct Idx {
    int v[10];
    uint4 g0, g1;
    int t1, t2;
    uint2 w;
  };
  __device__ __forceinline__ uint32_t pf_bytes(int64_t, int64_t) const { return PF_BYTES; }
  __device__ __forceinline__ void prefetch(int64_t tile, int64_t, uint8_t *dst,
                                           uint64_t *mbar) const {
    bulk_g2s(dst, blocks + tile * PF_BYTES, PF_BYTES, mbar);
  }
  __device__ __forceinline__ Idx load_idx(const uint8_t *pf, int r) const {
    Idx d;
    const int32_t *l = reinterpret_cast<const int32_t *>(pf + B_LST);
#pragma unroll
    for (int s = 0; s < 10; ++s) d.v[s] = l[128 * s + r];
    const uint4 *g = reinterpret_cast<const uint4 *>(pf + B_GEO + 32 * r);
    d.g0 = g[0];
    d.g1 = g[1];
    const int32_t *t = reinterpret_cast<const int32_t *>(pf + B_ESH);
    d.t1 = t[r];
    d.t2 = t[128 + r];
    d.w = reinterpret_cast<const uint2 *>(pf + B_EVS)[r];
    return d;
  }
  __device__ __forceinline__ float stage(int64_t, bool live, const Idx &d, uint4 (&c)[4]) const {
    float uv[10];
    float ss = 0.0f, qh = 0.0f;
    uint4 g0 = make_uint4(0, 0, 0, 0), g1 = g0;
    if (live) {
#pragma unroll
      for (int s = 0; s < 10; ++s) {
        const int k = (d.v[s] < 0 ? -d.v[s] : d.v[s]) - 1;
        const float uk = d.v[s] != 0 ? u[k] : 0.0f;
        uv[s] = d.v[s] < 0 ? -uk : uk;
      }
      const float q = 0.5f * (q_tr[d.t1] + q_tr[d.t2]);
      const float h = h_ref + 0.5f * (hd[d.w.x & 0x0FFFFFFFu] + hd[d.w.y & 0x0FFFFFFFu]);
#pragma unroll
      for (int s = 0; s < 10; ++s) ss += uv[s] * uv[s];
      qh = q * h;
      g0 = d.g0;
      g1 = d.g1;
    } else {
#pragma unroll
      for (int s = 0; s < 10; ++s) uv[s] = 0.0f;
    }
    const float sigma = sqrtf(ss * 0.1f) + 1e-30f;
    const float inv = 1.0f / sigma;
    c[0] = make_uint4(pack2(uv[0] * inv, uv[1] * inv), pack2(uv[2] * inv, uv[3] * inv),
                      pack2(uv[4] * inv, uv[5] * inv), pack2(uv[6] * inv, uv[7] * inv));
    c[1] = make_uint4(pack2(uv[8] * inv, uv[9] * inv), g0.x, g0.y, g0.z);
    c[2] = make_uint4(g0.w, g1.x, g1.y, g1.z);
    c[3] = make_uint4(0, 0, 0, 0);
    return qh * sigma;
  }
  __device__ __forceinline__ void write(int64_t e, float y, float qhs) const {
    corr[e] = qhs * fminf(fmaxf(y, -kCorrMax), kCorrMax);
  }
};

}  // namespace pipe
}  // namespace imodel
