// Learned surrogate force for hybrid HMC: the leapfrog integrates
//   -grad E(x)  ~  -(g_local(x) - F_nn(x)),
// where g_local is the exact gradient of the local penalty terms (area,
// volume, area difference, tether; FP32 stencils, one pass without the
// neighbour list) and F_nn is a message-passing network that stands in for
// the bending and repulsion forces.  Acceptance always uses the exact FP64
// Hamiltonian, so the chain samples the exact distribution; the surrogate
// only changes how often proposals are accepted.
//
// Network (width H = 64, SiLU, three rounds), per vertex i with ring j:
//   u_i   = 8 rotation-invariant vertex features (area, curvature, valence,
//           dihedral and edge-length statistics of the ring)
//   e_ij  = 4 edge features (length, dihedral, curvature difference / mean)
//   h_i   = SiLU(W_in u_i + b_in)
//   round r:  m_i = sum_j (W_e^r e_ij + b_e^r) * h_j          (gather, CUDA cores)
//             h_i = h_i + SiLU(W^r [h_i ; m_i] + b^r)          (tcgen05 BF16 GEMM)
//   F_i   = s ( sum_j c_ij (x_j - x_i)/|x_j - x_i| + c_i N_i ),
//           c_ij = sum_c w_o,c h_i,c h_j,c + b_o,  c_i = w_n . h_i + b_n,
//           N_i the area-weighted vertex normal.
// F is equivariant by construction (invariant coefficients on the edge
// directions and the normal).  Activations h, m are stored as bf16, the
// dense weights W^r are bf16 with FP32 accumulation in tensor memory; the
// small layers are FP32.
//
// The dense layer is one CTA per 128 vertices: TMA loads [h | m] (two
// 128 x 64 bf16 boxes) and W^r (two 64 x 64 boxes) into 128-byte-swizzled
// shared memory, one thread issues 8 tcgen05.mma (M 128, N 64, K 16), the
// accumulator (128 lanes x 64 FP32 columns) is read back by four warps and
// the epilogue adds bias, SiLU and the residual h (from the swizzled tile).
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

#include "tm_energy.cuh"
#include "tm_fp32.cuh"
#include "tm_internal.h"
#include "tm_math.cuh"
#include "tm_tc.cuh"

using namespace tmg;

#define TM_API_BEGIN try {
#define TM_API_END                  \
  }                                 \
  catch (const tmg::Error& e) {     \
    tmg::set_last_error(e.what());  \
    return e.code;                  \
  }                                 \
  catch (const std::exception& e) { \
    tmg::set_last_error(e.what());  \
    return TM_ERR_ARG;              \
  }                                 \
  return TM_OK;

namespace {

constexpr int H = 64, FV = 8, FE = 4, NR = 3, BM = 128;
constexpr int BLOB_HEADER = 8;
constexpr int BLOB_SIZE = BLOB_HEADER + H * FV + H + NR * (H * FE + H + H * 2 * H + H) + H + 1 + H + 1;

// FP32 parameters of the small layers (device copy)
struct SurW {
  float win[H * FV], bin[H];
  float we[NR][H * FE], be[NR][H], b[NR][H];
  float wo[H], wn[H];
  float bo, bn, lbar, abar, fscale;
};

}  // namespace

struct tm_surrogate {
  int nv = 0;
  SurW hw{};
  DevBuf<SurW> w;
  DevBuf<__nv_bfloat16> wd;  // dense weights [NR][H][2H] (row n, column k)
  DevBuf<float> u, nrm;
  DevBuf<__nv_bfloat16> hb[2], mb;
  DevBuf<double> gloc;
  DevBuf<int> status;
  alignas(64) CUtensorMap map_h[2];
  alignas(64) CUtensorMap map_m;
  alignas(64) CUtensorMap map_w[NR];
};

namespace {

using namespace tmg::fp32;
using tmg::tc::smem_u32;

inline int nblk(long n, int b) { return (int)((n + b - 1) / b); }

__device__ __forceinline__ float silu(float x) { return x / (1.0f + __expf(-x)); }

// vertex features, normal and embedding (one thread per vertex)
__global__ void k_sfeat(Topo t, const FaceF* __restrict__ fd, const EdgeF* __restrict__ ed,
                        const float* __restrict__ rho, const SurW* __restrict__ W, float* __restrict__ u,
                        float* __restrict__ nrm, __nv_bfloat16* __restrict__ h) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= t.nv) return;
  const float lbar = W->lbar, abar = W->abar;
  int d = t.val[i];
  float A = 0.f, ls = 0.f, l2 = 0.f, ths = 0.f, th2 = 0.f;
  f3 N = {0.f, 0.f, 0.f};
  for (int m = 0; m < d; ++m) {
    int4 s = t.slot[(size_t)m * t.nv + i];
    int f = slot_face(s.y);
    if (f >= 0) {
      FaceF F = fd[f];
      A += F.A;
      N += F.A * f3{F.nx, F.ny, F.nz};
    }
    EdgeF E = ed[s.z];
    float lr = E.l / lbar;
    ls += lr;
    l2 += lr * lr;
    ths += E.th;
    th2 += E.th * E.th;
  }
  float inv_d = d > 0 ? 1.0f / d : 0.0f;
  float x[FV];
  float rl = rho[i] * lbar;
  x[0] = (A / 3.0f) / abar - 1.0f;
  x[1] = rl;
  x[2] = rl * rl;
  x[3] = (d - 6) * (1.0f / 6.0f);
  x[4] = ths * inv_d;
  x[5] = sqrtf(th2 * inv_d);
  x[6] = ls * inv_d - 1.0f;
  x[7] = sqrtf(fmaxf(l2 * inv_d - (ls * inv_d) * (ls * inv_d), 0.0f));
  for (int k = 0; k < FV; ++k) u[(size_t)FV * i + k] = x[k];
  float nn = fnorm(N);
  float in = nn > 0.f ? 1.0f / nn : 0.0f;
  nrm[4 * (size_t)i] = N.x * in;
  nrm[4 * (size_t)i + 1] = N.y * in;
  nrm[4 * (size_t)i + 2] = N.z * in;
  nrm[4 * (size_t)i + 3] = 0.f;
  __nv_bfloat162* h2 = reinterpret_cast<__nv_bfloat162*>(h + (size_t)H * i);
  for (int c = 0; c < H; c += 2) {
    float y0 = W->bin[c], y1 = W->bin[c + 1];
    for (int k = 0; k < FV; ++k) {
      y0 += W->win[c * FV + k] * x[k];
      y1 += W->win[(c + 1) * FV + k] * x[k];
    }
    h2[c / 2] = __floats2bfloat162_rn(silu(y0), silu(y1));
  }
}

__device__ __forceinline__ void edge_feat(const EdgeF& E, float ri, float rj, float lbar, float* ef) {
  ef[0] = E.l / lbar - 1.0f;
  ef[1] = E.th;
  ef[2] = (rj - ri) * lbar;
  ef[3] = 0.5f * (rj + ri) * lbar;
}

__device__ __forceinline__ void unpack8(uint4 v, float* f) {
  const __nv_bfloat162* b = reinterpret_cast<const __nv_bfloat162*>(&v);
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    float2 x = __bfloat1622float2(b[q]);
    f[2 * q] = x.x;
    f[2 * q + 1] = x.y;
  }
}
__device__ __forceinline__ uint4 pack8(const float* f) {
  uint4 v;
  __nv_bfloat162* b = reinterpret_cast<__nv_bfloat162*>(&v);
#pragma unroll
  for (int q = 0; q < 4; ++q) b[q] = __floats2bfloat162_rn(f[2 * q], f[2 * q + 1]);
  return v;
}

// m_i = sum_j (W_e e_ij + b_e) * h_j: sixteen threads per vertex, four
// channels (8 bytes of h_j) per thread; the next ring slot is loaded while
// the current neighbour is summed
__global__ void __launch_bounds__(256) k_agg(Topo t, const EdgeF* __restrict__ ed, const float* __restrict__ rho,
                                             const SurW* __restrict__ W, int r, const __nv_bfloat16* __restrict__ h,
                                             __nv_bfloat16* __restrict__ mout) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = g >> 4, sub = g & 15;
  if (i >= t.nv) return;
  float4 w[4];
  float b[4];
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const int ch = 4 * sub + c;
    w[c] = *reinterpret_cast<const float4*>(&W->we[r][ch * FE]);
    b[c] = W->be[r][ch];
  }
  const float lbar = W->lbar, ri = rho[i];
  const uint2* h2 = reinterpret_cast<const uint2*>(h);
  float acc[4] = {0.f, 0.f, 0.f, 0.f};
  const int d = t.val[i];
  int4 s = d > 0 ? t.slot[i] : make_int4(0, 0, 0, 0);
  for (int m = 0; m < d; ++m) {
    const int4 sn = m + 1 < d ? t.slot[(size_t)(m + 1) * t.nv + i] : s;
    const int j = s.x;
    const uint2 hv = h2[(size_t)j * (H / 4) + sub];
    float ef[FE];
    edge_feat(ed[s.z], ri, rho[j], lbar, ef);
    const float2 h01 = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&hv.x));
    const float2 h23 = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&hv.y));
    const float hj[4] = {h01.x, h01.y, h23.x, h23.y};
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      float gt = b[c] + w[c].x * ef[0] + w[c].y * ef[1] + w[c].z * ef[2] + w[c].w * ef[3];
      acc[c] += gt * hj[c];
    }
    s = sn;
  }
  uint2 o;
  *reinterpret_cast<__nv_bfloat162*>(&o.x) = __floats2bfloat162_rn(acc[0], acc[1]);
  *reinterpret_cast<__nv_bfloat162*>(&o.y) = __floats2bfloat162_rn(acc[2], acc[3]);
  reinterpret_cast<uint2*>(mout)[(size_t)i * (H / 4) + sub] = o;
}

// h_out = h + SiLU([h | m] W^T + b) for 128 vertices per CTA on the tensor cores
constexpr int DENSE_SMEM = 1024 + 49152 + 64;

// Every wait is bounded: wait_polls polls for the tile loads and for the MMA
// completion.  When a wait gives up the CTA records it in *status (1 loads,
// 2 MMA), skips the work that depended on it, waits (with the long default
// limit) for the copies and the MMA it did issue to land, and frees its
// tensor memory before it returns.
constexpr int WAIT_POLLS = 1 << 22;
__global__ void __launch_bounds__(128) k_dense(const __grid_constant__ CUtensorMap mh,
                                               const __grid_constant__ CUtensorMap mm,
                                               const __grid_constant__ CUtensorMap mw, const float* __restrict__ bias,
                                               __nv_bfloat16* __restrict__ out, int M, int* status, int wait_polls,
                                               float* __restrict__ zout) {
  using namespace tmg::tc;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t* A0 = base;           // h tile, 128 rows x 128 B
  uint8_t* A1 = base + 16384;   // m tile
  uint8_t* B0 = base + 32768;   // W[:, 0:64], 64 rows x 128 B
  uint8_t* B1 = base + 40960;   // W[:, 64:128]
  uint64_t* bars = reinterpret_cast<uint64_t*>(base + 49152);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(base + 49152 + 16);
  int* issued = reinterpret_cast<int*>(base + 49152 + 20);  // the MMA was issued
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.x * BM;
  if (threadIdx.x == 0) {
    tma_prefetch_desc(&mh);
    tma_prefetch_desc(&mm);
    tma_prefetch_desc(&mw);
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    mbar_fence_init();
    *issued = 0;
  }
  if (warp == 0) {
    tmem_alloc(tslot, 64);
    tmem_relinquish();
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;
  if (threadIdx.x == 0) {
    mbar_expect_tx(&bars[0], 49152);
    tma_load_2d(A0, &mh, &bars[0], 0, m0);
    tma_load_2d(A1, &mm, &bars[0], 0, m0);
    tma_load_2d(B0, &mw, &bars[0], 0, 0);
    tma_load_2d(B1, &mw, &bars[0], 64, 0);
    if (mbar_wait(&bars[0], 0, wait_polls)) {
      tc_fence_after();
      constexpr uint32_t idesc = idesc_bf16_f32(BM, H);
#pragma unroll
      for (int kc = 0; kc < 2; ++kc) {
        const uint32_t a = smem_u32(kc ? A1 : A0), b = smem_u32(kc ? B1 : B0);
#pragma unroll
        for (int k = 0; k < 4; ++k)
          mma_bf16(tmem, sdesc_sw128(a + 32 * k, 1024), sdesc_sw128(b + 32 * k, 1024), idesc, (kc | k) != 0);
      }
      mma_commit(&bars[1]);
      *issued = 1;
    } else {
      atomicExch(status, 1);  // tile loads did not arrive in time
      // the copies are still this CTA's: let them land before it exits
      if (!mbar_wait(&bars[0], 0, WAIT_POLLS)) atomicExch(status, 3);
    }
  }
  __syncthreads();
  bool done = __all_sync(0xffffffffu, mbar_wait(&bars[1], 0, wait_polls));
  tc_fence_after();
  if (done) {
    const int r = warp * 32 + lane;
    float acc[H];
    const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16);
    tmem_ld32(taddr, acc);
    tmem_ld32(taddr + 32, acc + 32);
    if (m0 + r < M) {
      const uint8_t* rowp = A0 + (r >> 3) * 1024 + (r & 7) * 128;
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        uint4 hv = *reinterpret_cast<const uint4*>(rowp + ((c ^ (r & 7)) * 16));
        const __nv_bfloat162* h2 = reinterpret_cast<const __nv_bfloat162*>(&hv);
        uint4 ov;
        __nv_bfloat162* o2 = reinterpret_cast<__nv_bfloat162*>(&ov);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int n = c * 8 + 2 * q;
          float2 hf = __bfloat1622float2(h2[q]);
          const float z0 = acc[n] + bias[n], z1 = acc[n + 1] + bias[n + 1];
          o2[q] = __floats2bfloat162_rn(hf.x + silu(z0), hf.y + silu(z1));
          if (zout) *reinterpret_cast<float2*>(zout + (size_t)(m0 + r) * H + n) = make_float2(z0, z1);
        }
        *reinterpret_cast<uint4*>(out + (size_t)(m0 + r) * H + c * 8) = ov;
      }
    }
  } else {
    if (lane == 0) atomicExch(status, 2);  // the MMA completion did not arrive in time
    // an MMA that was issued still writes the accumulator: wait for it
    // before the tensor memory is freed
    if (threadIdx.x == 0 && *issued && !mbar_wait(&bars[1], 0, WAIT_POLLS)) atomicExch(status, 3);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, 64);
}

// output head: g = g_local - s (sum_j c_ij d_ij + c_i N_i), eight threads
// per vertex with eight channels each; the channel sums are reduced within
// the eight threads in a fixed order
__global__ void k_out(Topo t, Split S, const float* __restrict__ nrm, const SurW* __restrict__ W,
                      const __nv_bfloat16* __restrict__ h, const double* __restrict__ gloc, double* __restrict__ g) {
  const int gt = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = gt >> 3, sub = gt & 7;
  if (i >= t.nv) return;
  const unsigned gmask = 0xffu << (threadIdx.x & 24);  // the eight threads of this vertex
  const uint4* h4 = reinterpret_cast<const uint4*>(h);
  float hi[8], pi[8];
  unpack8(h4[(size_t)i * (H / 8) + sub], hi);
  float cn = 0.f;
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    pi[c] = W->wo[8 * sub + c] * hi[c];
    cn += W->wn[8 * sub + c] * hi[c];
  }
#pragma unroll
  for (int o = 1; o < 8; o <<= 1) cn += __shfl_xor_sync(gmask, cn, o);
  cn += W->bn;
  f3 F = cn * f3{nrm[4 * (size_t)i], nrm[4 * (size_t)i + 1], nrm[4 * (size_t)i + 2]};
  const float bo = W->bo;
  const int d = t.val[i];
  for (int m = 0; m < d; ++m) {
    const int j = t.nbr[(size_t)m * t.nv + i];
    float hj[8];
    unpack8(h4[(size_t)j * (H / 8) + sub], hj);
    float c = 0.f;
#pragma unroll
    for (int q = 0; q < 8; ++q) c += pi[q] * hj[q];
#pragma unroll
    for (int o = 1; o < 8; o <<= 1) c += __shfl_xor_sync(gmask, c, o);
    c += bo;
    f3 e = S.diff(j, i);
    F += (c / fnorm(e)) * e;
  }
  if (sub == 0) {
    const float sc = W->fscale;
    g[3 * (size_t)i] = gloc[3 * (size_t)i] - (double)(sc * F.x);
    g[3 * (size_t)i + 1] = gloc[3 * (size_t)i + 1] - (double)(sc * F.y);
    g[3 * (size_t)i + 2] = gloc[3 * (size_t)i + 2] - (double)(sc * F.z);
  }
}

// training inputs: ring neighbours, edge features and unit edge directions,
// slot-major [D][nv] (neighbour -1 and zeros past the valence)
__global__ void k_export(Topo t, Split S, const EdgeF* __restrict__ ed, const float* __restrict__ rho,
                         const SurW* __restrict__ W, int D, int* __restrict__ nbr, float* __restrict__ ef,
                         float* __restrict__ tv) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= t.nv) return;
  int d = t.val[i];
  for (int m = 0; m < D; ++m) {
    size_t o = (size_t)m * t.nv + i;
    float f[FE] = {0.f, 0.f, 0.f, 0.f};
    f3 dir = {0.f, 0.f, 0.f};
    int j = -1;
    if (m < d) {
      int4 s = t.slot[o];
      j = s.x;
      edge_feat(ed[s.z], rho[i], rho[j], W->lbar, f);
      f3 e = S.diff(j, i);
      dir = (1.0f / fnorm(e)) * e;
    }
    nbr[o] = j;
    for (int k = 0; k < FE; ++k) ef[FE * o + k] = f[k];
    tv[3 * o] = dir.x;
    tv[3 * o + 1] = dir.y;
    tv[3 * o + 2] = dir.z;
  }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    TM_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q));
    if (q != cudaDriverEntryPointSuccess || !p) fail(TM_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
    fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

// bf16 row-major [rows][cols] matrix, boxes of 64 columns x box_rows rows,
// 128-byte swizzle
void make_map(CUtensorMap* map, const void* ptr, uint64_t rows, uint64_t cols, uint32_t box_rows) {
  if ((reinterpret_cast<uintptr_t>(ptr) & 15) != 0) fail(TM_ERR_ARG, "tensor base not 16-byte aligned");
  cuuint64_t dims[2] = {cols, rows};
  cuuint64_t strides[1] = {cols * sizeof(__nv_bfloat16)};
  cuuint32_t box[2] = {64, box_rows};
  cuuint32_t es[2] = {1, 1};
  CUresult r = encode_fn()(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(ptr), dims, strides, box, es,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) fail(TM_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
}

void dense_launch(const CUtensorMap& mh, const CUtensorMap& mm, const CUtensorMap& mw, const float* bias,
                  __nv_bfloat16* out, int M, int* status, cudaStream_t s, int wait_polls = WAIT_POLLS,
                  float* zout = nullptr) {
  static bool attr = false;
  if (!attr) {
    TM_CUDA(cudaFuncSetAttribute(k_dense, cudaFuncAttributeMaxDynamicSharedMemorySize, DENSE_SMEM));
    attr = true;
  }
  if (M > 0) k_dense<<<nblk(M, BM), BM, DENSE_SMEM, s>>>(mh, mm, mw, bias, out, M, status, wait_polls, zout);
  TM_LAUNCH();
}

void parse_blob(const float* b, int64_t n, SurW& w, std::vector<__nv_bfloat16>& wd) {
  if (n != BLOB_SIZE) fail(TM_ERR_ARG, "surrogate weights: expected " + std::to_string(BLOB_SIZE) + " floats");
  if (b[0] != 1.0f || b[1] != FV || b[2] != FE || b[3] != H || b[4] != NR)
    fail(TM_ERR_ARG, "surrogate weights: unsupported layout");
  w.lbar = b[5];
  w.abar = b[6];
  w.fscale = b[7];
  if (!(w.lbar > 0) || !(w.abar > 0)) fail(TM_ERR_ARG, "surrogate weights: non-positive length or area scale");
  const float* q = b + BLOB_HEADER;
  auto take = [&](float* dst, int k) {
    std::memcpy(dst, q, sizeof(float) * k);
    q += k;
  };
  take(w.win, H * FV);
  take(w.bin, H);
  wd.resize((size_t)NR * H * 2 * H);
  for (int r = 0; r < NR; ++r) {
    take(w.we[r], H * FE);
    take(w.be[r], H);
    for (int k = 0; k < H * 2 * H; ++k) wd[(size_t)r * H * 2 * H + k] = __float2bfloat16_rn(q[k]);
    q += H * 2 * H;
    take(w.b[r], H);
  }
  take(w.wo, H);
  take(&w.bo, 1);
  take(w.wn, H);
  take(&w.bn, 1);
}

}  // namespace

namespace tmg {

// surrogate gradient at positions P into g (device arrays of 3 nv doubles)
void surrogate_grad(tm_surrogate* sg, tm_energy* e, tm_mesh* m, const double* P, double* g, cudaStream_t s) {
  if (m->nv != sg->nv) fail(TM_ERR_ARG, "surrogate built for another mesh size");
  int nv = m->nv;
  if (nv == 0) return;
  energy_eval32_local(e, m, P, sg->gloc.get(), s);
  Topo t = m->topo();
  const FaceF* fd = reinterpret_cast<const FaceF*>(e->face.get());
  const EdgeF* ed = reinterpret_cast<const EdgeF*>(e->edge.get());
  const float* rho = reinterpret_cast<const float*>(e->rho.get());
  Split S{e->pos32.get(), e->poslo.get()};
  SurW* W = sg->w.get();
  k_sfeat<<<nblk(nv, 128), 128, 0, s>>>(t, fd, ed, rho, W, sg->u.get(), sg->nrm.get(), sg->hb[0].get());
  TM_LAUNCH();
  int cur = 0;
  for (int r = 0; r < NR; ++r) {
    k_agg<<<nblk(16L * nv, 256), 256, 0, s>>>(t, ed, rho, W, r, sg->hb[cur].get(), sg->mb.get());
    TM_LAUNCH();
    dense_launch(sg->map_h[cur], sg->map_m, sg->map_w[r], W->b[r], sg->hb[cur ^ 1].get(), nv, sg->status.get(), s);
    cur ^= 1;
  }
  k_out<<<nblk(8L * nv, 256), 256, 0, s>>>(t, S, sg->nrm.get(), W, sg->hb[cur].get(), sg->gloc.get(), g);
  TM_LAUNCH();
}

}  // namespace tmg

// --------------------------------------------------------------------------
// Training on the GPU: hand-written forward and backward kernels of the
// network above and Adam, on the inputs tm_surrogate_inputs_device exports.
//
// Parameters live as one FP32 vector theta in the blob's order (the
// header dropped).  The forward pass is the inference pass with its
// intermediates kept: h and m in bf16 (as the inference kernels store
// them), the dense weights rounded to bf16 with FP32 accumulation (the
// same tcgen05 layer, which also writes the pre-activations z in FP32).
// The backward pass treats the bf16 roundings as identities (straight
// through) and accumulates in FP32:
//   output   dF_i = 2 (F_i - T_i) / (3 n rms^2),  dc_ij = s dF_i . d_ij,
//            dc_i = s dF_i . N_i,  dh_i = dc_i w_n + w_o * sum_j (dc_ij + dc_ji) h_j
//   dense    dz = dh * SiLU'(z), d[h ; m] = dz W (h part added to the
//            residual), dW += dz [h ; m]^T, db += dz
//   messages dh_j += sum_i (W_e e_ij + b_e) * dm_i over the rings of j,
//            dW_e += (dm_i * h_j) e_ij^T, db_e += dm_i * h_j
//   input    dz = dh * SiLU'(z), dW_in += dz u^T, db_in += dz
// Parameter gradients are summed per block and then over the blocks in
// block order (no floating-point atomics: a step is bit-reproducible).
// --------------------------------------------------------------------------
namespace {

// offsets of the parameter groups in theta
constexpr int P_WIN = 0, P_BIN = H * FV, P_R0 = P_BIN + H;
constexpr int P_RSTRIDE = H * FE + H + H * 2 * H + H;
__host__ __device__ constexpr int p_we(int r) { return P_R0 + r * P_RSTRIDE; }
__host__ __device__ constexpr int p_be(int r) { return p_we(r) + H * FE; }
__host__ __device__ constexpr int p_w(int r) { return p_be(r) + H; }
__host__ __device__ constexpr int p_b(int r) { return p_w(r) + H * 2 * H; }
constexpr int P_WO = P_R0 + NR * P_RSTRIDE, P_BO = P_WO + H, P_WN = P_BO + 1, P_BN = P_WN + H;
constexpr int NPARAM = P_BN + 1;
static_assert(NPARAM + BLOB_HEADER == BLOB_SIZE, "parameter layout");

__device__ __forceinline__ float dsilu(float z) {
  const float sg = 1.0f / (1.0f + __expf(-z));
  return sg * (1.0f + z * (1.0f - sg));
}

constexpr int TB = 256;  // threads per block of the per-vertex training kernels

// input layer: z = W_in u + b_in, h = bf16(SiLU(z)); 8 threads per vertex,
// 8 channels each
__global__ void __launch_bounds__(TB) k_t_embed(int nv, const float* __restrict__ u, const float* __restrict__ th,
                                                float* __restrict__ z, __nv_bfloat16* __restrict__ h) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = g >> 3, sub = g & 7;
  if (i >= nv) return;
  float x[FV];
#pragma unroll
  for (int k = 0; k < FV; ++k) x[k] = u[(size_t)FV * i + k];
  float o[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const int c = 8 * sub + q;
    float y = th[P_BIN + c];
#pragma unroll
    for (int k = 0; k < FV; ++k) y += th[P_WIN + c * FV + k] * x[k];
    z[(size_t)H * i + c] = y;
    o[q] = silu(y);
  }
  reinterpret_cast<uint4*>(h)[(size_t)i * (H / 8) + sub] = pack8(o);
}

// messages m_i = sum_j (W_e e_ij + b_e) * h_j over the exported rings
// (nbr / ef slot-major [D][n]); 16 threads per vertex, 4 channels each
__global__ void __launch_bounds__(TB) k_t_agg(int nv, int D, const int* __restrict__ nbr, const float* __restrict__ ef,
                                              const float* __restrict__ th, int r,
                                              const __nv_bfloat16* __restrict__ h, __nv_bfloat16* __restrict__ mout) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = g >> 4, sub = g & 15;
  if (i >= nv) return;
  float4 w[4];
  float b[4];
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const int ch = 4 * sub + c;
    w[c] = *reinterpret_cast<const float4*>(th + p_we(r) + ch * FE);
    b[c] = th[p_be(r) + ch];
  }
  const uint2* h2 = reinterpret_cast<const uint2*>(h);
  float acc[4] = {0.f, 0.f, 0.f, 0.f};
  for (int m = 0; m < D; ++m) {
    const size_t o = (size_t)m * nv + i;
    const int j = nbr[o];
    if (j < 0) break;
    const float4 e = *reinterpret_cast<const float4*>(ef + FE * o);
    const uint2 hv = h2[(size_t)j * (H / 4) + sub];
    const float2 h01 = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&hv.x));
    const float2 h23 = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&hv.y));
    const float hj[4] = {h01.x, h01.y, h23.x, h23.y};
#pragma unroll
    for (int c = 0; c < 4; ++c) acc[c] += (b[c] + w[c].x * e.x + w[c].y * e.y + w[c].z * e.z + w[c].w * e.w) * hj[c];
  }
  uint2 o;
  *reinterpret_cast<__nv_bfloat162*>(&o.x) = __floats2bfloat162_rn(acc[0], acc[1]);
  *reinterpret_cast<__nv_bfloat162*>(&o.y) = __floats2bfloat162_rn(acc[2], acc[3]);
  reinterpret_cast<uint2*>(mout)[(size_t)i * (H / 4) + sub] = o;
}

// Sum of a per-thread value over the block's threads in thread order,
// through shared memory (deterministic); returns it in thread 0.
__device__ __forceinline__ float block_sum(float v, float* sh) {
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  const float r = sh[0];
  __syncthreads();
  return r;
}

// Per-channel sums over the vertices of a block, where thread t holds
// channels 8 (t & 7) .. 8 (t & 7) + 7 of vertex t >> 3 (32 vertices): the
// column sums in vertex order into out[0..63].
__device__ __forceinline__ void block_channel_sum(const float* v8, float* sh, float* out) {
  const int sub = threadIdx.x & 7, vi = threadIdx.x >> 3;
#pragma unroll
  for (int q = 0; q < 8; ++q) sh[vi * H + 8 * sub + q] = v8[q];
  __syncthreads();
  if (threadIdx.x < H) {
    float s = 0.f;
    for (int k = 0; k < TB / 8; ++k) s += sh[k * H + threadIdx.x];
    out[threadIdx.x] = s;
  }
  __syncthreads();
}

// output head, loss and dL/dF: 8 threads per vertex
__global__ void __launch_bounds__(TB) k_t_out(int nv, int D, const int* __restrict__ nbr,
                                              const float* __restrict__ dirs, const float* __restrict__ nrm,
                                              const float* __restrict__ tgt, const float* __restrict__ th, float fs,
                                              float inv_norm, const __nv_bfloat16* __restrict__ h,
                                              float* __restrict__ F, float* __restrict__ dF,
                                              float* __restrict__ lossp) {
  __shared__ float sh[TB];
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = g >> 3, sub = g & 7;
  const unsigned gmask = 0xffu << (threadIdx.x & 24);
  const bool act = i < nv;
  const int ii = act ? i : 0;
  const uint4* h4 = reinterpret_cast<const uint4*>(h);
  float hi[8], pi[8];
  unpack8(h4[(size_t)ii * (H / 8) + sub], hi);
  float cn = 0.f;
#pragma unroll
  for (int c = 0; c < 8; ++c) {
    pi[c] = th[P_WO + 8 * sub + c] * hi[c];
    cn += th[P_WN + 8 * sub + c] * hi[c];
  }
#pragma unroll
  for (int o = 1; o < 8; o <<= 1) cn += __shfl_xor_sync(gmask, cn, o);
  cn += th[P_BN];
  float Fx = cn * nrm[4 * (size_t)ii], Fy = cn * nrm[4 * (size_t)ii + 1], Fz = cn * nrm[4 * (size_t)ii + 2];
  const float bo = th[P_BO];
  for (int m = 0; m < D; ++m) {
    const size_t o = (size_t)m * nv + ii;
    const int j = nbr[o];
    if (j < 0) break;
    float hj[8];
    unpack8(h4[(size_t)j * (H / 8) + sub], hj);
    float c = 0.f;
#pragma unroll
    for (int q = 0; q < 8; ++q) c += pi[q] * hj[q];
#pragma unroll
    for (int q = 1; q < 8; q <<= 1) c += __shfl_xor_sync(gmask, c, q);
    c += bo;
    Fx += c * dirs[3 * o];
    Fy += c * dirs[3 * o + 1];
    Fz += c * dirs[3 * o + 2];
  }
  Fx *= fs;
  Fy *= fs;
  Fz *= fs;
  float l = 0.f;
  if (act && sub == 0) {
    const float ex = Fx - tgt[3 * (size_t)i], ey = Fy - tgt[3 * (size_t)i + 1], ez = Fz - tgt[3 * (size_t)i + 2];
    l = (ex * ex + ey * ey + ez * ez) * inv_norm;
    if (F) {
      F[3 * (size_t)i] = Fx;
      F[3 * (size_t)i + 1] = Fy;
      F[3 * (size_t)i + 2] = Fz;
    }
    dF[3 * (size_t)i] = 2.0f * inv_norm * ex;
    dF[3 * (size_t)i + 1] = 2.0f * inv_norm * ey;
    dF[3 * (size_t)i + 2] = 2.0f * inv_norm * ez;
  }
  const float s = block_sum(l, sh);
  if (threadIdx.x == 0) lossp[blockIdx.x] = s;
}

// Backward of the output head: dh of the last round (FP32) and the block
// partials of (w_o, b_o, w_n, b_n) (part: 130 floats per block)
__global__ void __launch_bounds__(TB) k_t_outback(int nv, int D, const int* __restrict__ nbr,
                                                  const float* __restrict__ dirs, const float* __restrict__ nrm,
                                                  const float* __restrict__ th, float fs,
                                                  const __nv_bfloat16* __restrict__ h, const float* __restrict__ dF,
                                                  float* __restrict__ dh, float* __restrict__ part) {
  __shared__ float sh[(TB / 8) * H];
  __shared__ float sred[TB];
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = g >> 3, sub = g & 7;
  const bool act = i < nv;
  const int ii = act ? i : 0;
  const uint4* h4 = reinterpret_cast<const uint4*>(h);
  float hi[8], acc[8], pwo[8], pwn[8];
  unpack8(h4[(size_t)ii * (H / 8) + sub], hi);
  const float dfx = act ? dF[3 * (size_t)ii] : 0.f, dfy = act ? dF[3 * (size_t)ii + 1] : 0.f,
              dfz = act ? dF[3 * (size_t)ii + 2] : 0.f;
  const float dci = fs * (dfx * nrm[4 * (size_t)ii] + dfy * nrm[4 * (size_t)ii + 1] + dfz * nrm[4 * (size_t)ii + 2]);
  float pbo = 0.f;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    acc[q] = dci * th[P_WN + 8 * sub + q];
    pwn[q] = dci * hi[q];
    pwo[q] = 0.f;
  }
  for (int m = 0; act && m < D; ++m) {
    const size_t o = (size_t)m * nv + ii;
    const int j = nbr[o];
    if (j < 0) break;
    const float ux = dirs[3 * o], uy = dirs[3 * o + 1], uz = dirs[3 * o + 2];
    const float dcij = fs * (dfx * ux + dfy * uy + dfz * uz);
    const float dcji = -fs * (dF[3 * (size_t)j] * ux + dF[3 * (size_t)j + 1] * uy + dF[3 * (size_t)j + 2] * uz);
    float hj[8];
    unpack8(h4[(size_t)j * (H / 8) + sub], hj);
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      acc[q] += (dcij + dcji) * th[P_WO + 8 * sub + q] * hj[q];
      pwo[q] += dcij * hi[q] * hj[q];
    }
    if (sub == 0) pbo += dcij;
  }
  if (act)
#pragma unroll
    for (int q = 0; q < 8; ++q) dh[(size_t)H * i + 8 * sub + q] = acc[q];
  float* pb = part + 130 * (size_t)blockIdx.x;
  block_channel_sum(pwo, sh, pb);
  block_channel_sum(pwn, sh, pb + 65);
  const float sbo = block_sum(pbo, sred);
  const float sbn = block_sum(sub == 0 ? dci : 0.f, sred);
  if (threadIdx.x == 0) {
    pb[64] = sbo;
    pb[129] = sbn;
  }
}

// Backward of dense layer r over tiles of 64 vertices (persistent blocks):
// dz = dh1 * SiLU'(z); dh0 = dh1 + dz W[:, :64]; dm = dz W[:, 64:];
// block partials of dW (64 x 128, row n, column k) and db (64).  Thread t
// owns column k = t & 127 and half of the rows (vertices for d[h | m],
// output channels for dW): shared-memory reads of W and [h | m] are
// consecutive across a warp, those of dz are broadcasts.
constexpr int DT = 64;  // vertices per tile
constexpr int DENSE_BACK_SMEM = (DT * H + DT * 2 * H + H * 2 * H) * sizeof(float);
__global__ void __launch_bounds__(TB) k_t_dense_back(int nv, const float* __restrict__ th, int r,
                                                     const float* __restrict__ z, const __nv_bfloat16* __restrict__ h,
                                                     const __nv_bfloat16* __restrict__ mm,
                                                     const float* __restrict__ dh1, float* __restrict__ dh0,
                                                     float* __restrict__ dm, float* __restrict__ part) {
  extern __shared__ float sm[];
  float* sdz = sm;              // [DT][H]
  float* sa = sdz + DT * H;     // [DT][2H]: [h | m]
  float* sw = sa + DT * 2 * H;  // [H][2H]: W rounded to bf16
  const int t = threadIdx.x;
  const int k = t & (2 * H - 1), half = t >> 7;  // column, and rows half * 32 .. + 31
  for (int q = t; q < H * 2 * H; q += TB) sw[q] = __bfloat162float(__float2bfloat16_rn(th[p_w(r) + q]));
  float gw[32];
#pragma unroll
  for (int q = 0; q < 32; ++q) gw[q] = 0.f;
  float gb = 0.f;
  const int ntile = (nv + DT - 1) / DT;
  for (int tile = blockIdx.x; tile < ntile; tile += gridDim.x) {
    const int v0 = tile * DT;
    __syncthreads();  // the previous tile's reads are done (and sw is written)
    for (int q = t; q < DT * H; q += TB) {
      const int v = v0 + q / H;
      sdz[q] = v < nv ? dh1[(size_t)v0 * H + q] * dsilu(z[(size_t)v0 * H + q]) : 0.f;
    }
    for (int q = t; q < DT * 2 * H; q += TB) {
      const int vr = q / (2 * H), c = q % (2 * H), v = v0 + vr;
      float a = 0.f;
      if (v < nv) a = __bfloat162float(c < H ? h[(size_t)v * H + c] : mm[(size_t)v * H + c - H]);
      sa[q] = a;
    }
    __syncthreads();
    // d[h | m][v][k] = sum_n dz[v][n] W[n][k] for this thread's 32 vertices
    {
      float o[32];
#pragma unroll
      for (int q = 0; q < 32; ++q) o[q] = 0.f;
      for (int n = 0; n < H; ++n) {
        const float w = sw[n * 2 * H + k];
#pragma unroll
        for (int q = 0; q < 32; ++q) o[q] += sdz[(half * 32 + q) * H + n] * w;
      }
#pragma unroll
      for (int q = 0; q < 32; ++q) {
        const int v = v0 + half * 32 + q;
        if (v >= nv) break;
        if (k < H)
          dh0[(size_t)v * H + k] = dh1[(size_t)v * H + k] + o[q];
        else
          dm[(size_t)v * H + k - H] = o[q];
      }
    }
    // dW[n][k] += sum over the tile's vertices of dz[v][n] a[v][k], rows
    // n = half * 32 .. + 31
    for (int vr = 0; vr < DT; ++vr) {
      const float a = sa[vr * 2 * H + k];
#pragma unroll
      for (int q = 0; q < 32; ++q) gw[q] += sdz[vr * H + half * 32 + q] * a;
    }
    if (t < H)
      for (int vr = 0; vr < DT; ++vr) gb += sdz[vr * H + t];
  }
  float* pb = part + (size_t)(H * 2 * H + H) * blockIdx.x;
#pragma unroll
  for (int q = 0; q < 32; ++q) pb[(half * 32 + q) * 2 * H + k] = gw[q];
  if (t < H) pb[H * 2 * H + t] = gb;
}

// Backward of the messages of round r, per vertex v (16 threads, 4
// channels each): as a sender dh[v] += sum_i (W_e e_iv + b_e) * dm_i over
// v's ring (e_iv is e_vi with the antisymmetric feature 2 negated); as a
// receiver the block partials of dW_e and db_e (320 floats per block).
__global__ void __launch_bounds__(TB) k_t_msg_back(int nv, int D, const int* __restrict__ nbr,
                                                   const float* __restrict__ ef, const float* __restrict__ th, int r,
                                                   const __nv_bfloat16* __restrict__ h, const float* __restrict__ dm,
                                                   float* __restrict__ dh, float* __restrict__ part) {
  __shared__ float sh[TB];
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = g >> 4, sub = g & 15;
  const bool act = i < nv;
  const int ii = act ? i : 0;
  float4 w[4];
  float b[4], dmi[4], add[4] = {0.f, 0.f, 0.f, 0.f}, gwe[4][FE], gbe[4];
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const int ch = 4 * sub + c;
    w[c] = *reinterpret_cast<const float4*>(th + p_we(r) + ch * FE);
    b[c] = th[p_be(r) + ch];
    dmi[c] = dm[(size_t)H * ii + ch];
    gbe[c] = 0.f;
#pragma unroll
    for (int k = 0; k < FE; ++k) gwe[c][k] = 0.f;
  }
  const uint2* h2 = reinterpret_cast<const uint2*>(h);
  for (int m = 0; act && m < D; ++m) {
    const size_t o = (size_t)m * nv + ii;
    const int j = nbr[o];
    if (j < 0) break;
    const float4 e = *reinterpret_cast<const float4*>(ef + FE * o);  // e_vj
    const uint2 hv = h2[(size_t)j * (H / 4) + sub];
    const float2 h01 = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&hv.x));
    const float2 h23 = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&hv.y));
    const float hj[4] = {h01.x, h01.y, h23.x, h23.y};
    const float4 dmj = *reinterpret_cast<const float4*>(dm + (size_t)H * j + 4 * sub);
    const float dj[4] = {dmj.x, dmj.y, dmj.z, dmj.w};
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      // receiver: m_v gathers (W_e e_vj + b_e) * h_j
      const float q = dmi[c] * hj[c];
      gbe[c] += q;
      gwe[c][0] += q * e.x;
      gwe[c][1] += q * e.y;
      gwe[c][2] += q * e.z;
      gwe[c][3] += q * e.w;
      // sender: m_j gathers (W_e e_jv + b_e) * h_v, e_jv = e_vj with feature 2 negated
      add[c] += (b[c] + w[c].x * e.x + w[c].y * e.y - w[c].z * e.z + w[c].w * e.w) * dj[c];
    }
  }
  if (act) {
    float4* d4 = reinterpret_cast<float4*>(dh + (size_t)H * i + 4 * sub);
    float4 cur = *d4;
    cur.x += add[0];
    cur.y += add[1];
    cur.z += add[2];
    cur.w += add[3];
    *d4 = cur;
  }
  // block partials: thread (vertex, sub) holds 4 channels x (4 + 1) values;
  // sum over the block's 16 vertices per channel in vertex order
  float* pb = part + (H * FE + H) * (size_t)blockIdx.x;
  for (int k = 0; k < FE + 1; ++k) {
    for (int c = 0; c < 4; ++c) {
      sh[threadIdx.x] = k < FE ? gwe[c][k] : gbe[c];
      __syncthreads();
      if (threadIdx.x < 16) {
        float s = 0.f;
        for (int v = 0; v < TB / 16; ++v) s += sh[v * 16 + threadIdx.x];
        const int ch = 4 * threadIdx.x + c;
        if (k < FE)
          pb[ch * FE + k] = s;
        else
          pb[H * FE + ch] = s;
      }
      __syncthreads();
    }
  }
}

// Backward of the input layer: dz = dh * SiLU'(z), block partials of
// dW_in (64 x 8) and db_in (576 floats per block); 8 threads per vertex
__global__ void __launch_bounds__(TB) k_t_embed_back(int nv, const float* __restrict__ u, const float* __restrict__ z,
                                                     const float* __restrict__ dh, float* __restrict__ part) {
  __shared__ float sh[(TB / 8) * H];
  __shared__ float col[H];
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = g >> 3, sub = g & 7;
  const bool act = i < nv;
  const int ii = act ? i : 0;
  float x[FV], dz[8];
#pragma unroll
  for (int k = 0; k < FV; ++k) x[k] = act ? u[(size_t)FV * ii + k] : 0.f;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const size_t o = (size_t)H * ii + 8 * sub + q;
    dz[q] = act ? dh[o] * dsilu(z[o]) : 0.f;
  }
  float* pb = part + (H * FV + H) * (size_t)blockIdx.x;
  float v8[8];
  for (int k = 0; k < FV; ++k) {
#pragma unroll
    for (int q = 0; q < 8; ++q) v8[q] = dz[q] * x[k];
    block_channel_sum(v8, sh, col);
    if (threadIdx.x < H) pb[threadIdx.x * FV + k] = col[threadIdx.x];
  }
  block_channel_sum(dz, sh, col);
  if (threadIdx.x < H) pb[H * FV + threadIdx.x] = col[threadIdx.x];
}

// grad[dst + k] = sum over nb blocks (in block order) of part[b * stride + k]
__global__ void k_t_reduce(const float* __restrict__ part, int nb, int stride, int n, float* __restrict__ grad,
                           int dst) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  float s = 0.f;
  for (int b = 0; b < nb; ++b) s += part[(size_t)b * stride + k];
  grad[dst + k] = s;
}
// the output head's partials: (w_o 64, b_o 1, w_n 64, b_n 1) map onto
// theta's last 130 entries in the same order
__global__ void k_t_loss(const float* __restrict__ lossp, int nb, float* __restrict__ loss) {
  if (threadIdx.x || blockIdx.x) return;
  float s = 0.f;
  for (int b = 0; b < nb; ++b) s += lossp[b];
  *loss = s;
}

// Adam (Kingma & Ba 2015) with bias correction; the dense weights' bf16
// copies (what the forward reads) are refreshed from the FP32 master
__global__ void k_t_adam(int n, float* __restrict__ th, const float* __restrict__ g, float* __restrict__ m1,
                         float* __restrict__ m2, float lr, float b1, float b2, float eps, float c1, float c2,
                         __nv_bfloat16* __restrict__ wd) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const float gk = g[k];
  const float a = b1 * m1[k] + (1.0f - b1) * gk;
  const float b = b2 * m2[k] + (1.0f - b2) * gk * gk;
  m1[k] = a;
  m2[k] = b;
  const float x = th[k] - lr * (a * c1) / (sqrtf(b * c2) + eps);
  th[k] = x;
  for (int r = 0; r < NR; ++r)
    if (k >= p_w(r) && k < p_w(r) + H * 2 * H) wd[(size_t)r * H * 2 * H + (k - p_w(r))] = __float2bfloat16_rn(x);
}

}  // namespace

struct tm_strain {
  int nv = 0, D = 0;
  float lbar = 1.f, abar = 1.f, fscale = 1.f;
  long long step = 0;
  DevBuf<float> th, grad, m1, m2, loss;
  DevBuf<__nv_bfloat16> wd;      // [NR][H][2H]
  DevBuf<float> z;               // [NR + 1][nv][H]: input layer, then the dense layers
  DevBuf<__nv_bfloat16> hb;      // [NR + 1][nv][H]
  DevBuf<__nv_bfloat16> mb;      // [NR][nv][H]
  DevBuf<float> dha, dhb, dm, dF, part, lossp;
  DevBuf<int> status;
  int nb_dense = 0;
  alignas(64) CUtensorMap map_h[NR];
  alignas(64) CUtensorMap map_m[NR];
  alignas(64) CUtensorMap map_w[NR];
};

namespace {

int dense_back_blocks() {
  static int nbk = 0;
  if (!nbk) {
    TM_CUDA(cudaFuncSetAttribute(k_t_dense_back, cudaFuncAttributeMaxDynamicSharedMemorySize, DENSE_BACK_SMEM));
    int per_sm = 0, nsm = 0, dev = 0;
    TM_CUDA(cudaGetDevice(&dev));
    TM_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    TM_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_t_dense_back, TB, DENSE_BACK_SMEM));
    nbk = std::max(1, per_sm) * nsm;
  }
  return nbk;
}

struct TrainInputs {
  const float *u, *nrm, *ef, *dirs, *tgt;
  const int* nbr;
  int D;  // ring slots of the exported arrays ([D][n])
};

// forward pass (kept intermediates) and, with want_grad, the backward pass
// and the gradient into st->grad; F (n x 3, may be NULL) receives the force
void train_pass(tm_strain* st, const TrainInputs& in, float inv_norm, bool want_grad, float* F, cudaStream_t s) {
  const int nv = st->nv, D = in.D;
  const size_t NH = (size_t)nv * H;
  const float* th = st->th.get();
  const int nb8 = nblk((long)nv * 8, TB), nb16 = nblk((long)nv * 16, TB);
  k_t_embed<<<nb8, TB, 0, s>>>(nv, in.u, th, st->z.get(), st->hb.get());
  TM_LAUNCH();
  for (int r = 0; r < NR; ++r) {
    k_t_agg<<<nb16, TB, 0, s>>>(nv, D, in.nbr, in.ef, th, r, st->hb.get() + r * NH, st->mb.get() + r * NH);
    TM_LAUNCH();
    dense_launch(st->map_h[r], st->map_m[r], st->map_w[r], th + p_b(r), st->hb.get() + (r + 1) * NH, nv,
                 st->status.get(), s, WAIT_POLLS, st->z.get() + (r + 1) * NH);
  }
  k_t_out<<<nb8, TB, 0, s>>>(nv, D, in.nbr, in.dirs, in.nrm, in.tgt, th, st->fscale, inv_norm,
                              st->hb.get() + NR * NH, F, st->dF.get(), st->lossp.get());
  TM_LAUNCH();
  k_t_loss<<<1, 1, 0, s>>>(st->lossp.get(), nb8, st->loss.get());
  TM_LAUNCH();
  if (!want_grad) return;
  float* g = st->grad.get();
  float* part = st->part.get();
  // output head
  k_t_outback<<<nb8, TB, 0, s>>>(nv, D, in.nbr, in.dirs, in.nrm, th, st->fscale, st->hb.get() + NR * NH,
                                  st->dF.get(), st->dha.get(), part);
  TM_LAUNCH();
  k_t_reduce<<<1, 256, 0, s>>>(part, nb8, 130, 130, g, P_WO);
  TM_LAUNCH();
  // rounds, last to first: dense layer, then messages
  float* dcur = st->dha.get();
  float* dnext = st->dhb.get();
  const int nbd = st->nb_dense;
  for (int r = NR - 1; r >= 0; --r) {
    k_t_dense_back<<<nbd, TB, DENSE_BACK_SMEM, s>>>(nv, th, r, st->z.get() + (r + 1) * NH, st->hb.get() + r * NH,
                                                     st->mb.get() + r * NH, dcur, dnext, st->dm.get(), part);
    TM_LAUNCH();
    k_t_reduce<<<nblk(H * 2 * H + H, 256), 256, 0, s>>>(part, nbd, H * 2 * H + H, H * 2 * H, g, p_w(r));
    TM_LAUNCH();
    k_t_reduce<<<1, 256, 0, s>>>(part + H * 2 * H, nbd, H * 2 * H + H, H, g, p_b(r));
    TM_LAUNCH();
    k_t_msg_back<<<nb16, TB, 0, s>>>(nv, D, in.nbr, in.ef, th, r, st->hb.get() + r * NH, st->dm.get(), dnext, part);
    TM_LAUNCH();
    k_t_reduce<<<nblk(H * FE + H, 256), 256, 0, s>>>(part, nb16, H * FE + H, H * FE + H, g, p_we(r));
    TM_LAUNCH();
    std::swap(dcur, dnext);
  }
  // input layer
  k_t_embed_back<<<nb8, TB, 0, s>>>(nv, in.u, st->z.get(), dcur, part);
  TM_LAUNCH();
  k_t_reduce<<<nblk(H * FV + H, 256), 256, 0, s>>>(part, nb8, H * FV + H, H * FV + H, g, P_WIN);
  TM_LAUNCH();
}

TrainInputs check_inputs(tm_strain* st, int64_t nv, int32_t D, const float* u, const float* nrm, const int32_t* nbr,
                         const float* ef, const float* dirs, const float* tgt) {
  if (!st || !u || !nrm || !nbr || !ef || !dirs || !tgt) fail(TM_ERR_ARG, "NULL argument");
  if (nv != st->nv) fail(TM_ERR_ARG, "training state built for " + std::to_string(st->nv) + " vertices");
  if (D < 1 || D > st->D) fail(TM_ERR_ARG, "max_valence out of the training state's range");
  if ((reinterpret_cast<uintptr_t>(ef) & 15) != 0) fail(TM_ERR_ARG, "edge features not 16-byte aligned");
  TrainInputs in{u, nrm, ef, dirs, tgt, nbr, (int)D};
  return in;
}

}  // namespace

extern "C" {

int tm_surrogate_create(tm_mesh* m, const float* weights, int64_t n_weights, tm_surrogate** out) {
  TM_API_BEGIN
  if (!m || !weights || !out) fail(TM_ERR_ARG, "NULL argument");
  *out = nullptr;
  std::unique_ptr<tm_surrogate> sg(new tm_surrogate());
  std::vector<__nv_bfloat16> wd;
  parse_blob(weights, n_weights, sg->hw, wd);
  int nv = m->nv;
  sg->nv = nv;
  size_t n = std::max(nv, 1);
  sg->w.ensure(1);
  sg->wd.ensure(wd.size());
  sg->u.ensure(FV * n);
  sg->nrm.ensure(4 * n);
  sg->hb[0].ensure(H * n);
  sg->hb[1].ensure(H * n);
  sg->mb.ensure(H * n);
  sg->gloc.ensure(3 * n);
  sg->status.ensure(1);
  TM_CUDA(cudaMemcpy(sg->w.get(), &sg->hw, sizeof(SurW), cudaMemcpyHostToDevice));
  TM_CUDA(cudaMemcpy(sg->wd.get(), wd.data(), sizeof(__nv_bfloat16) * wd.size(), cudaMemcpyHostToDevice));
  TM_CUDA(cudaMemset(sg->status.get(), 0, sizeof(int)));
  if (nv > 0) {
    for (int k = 0; k < 2; ++k) make_map(&sg->map_h[k], sg->hb[k].get(), nv, H, BM);
    make_map(&sg->map_m, sg->mb.get(), nv, H, BM);
  }
  for (int r = 0; r < NR; ++r) make_map(&sg->map_w[r], sg->wd.get() + (size_t)r * H * 2 * H, H, 2 * H, H);
  *out = sg.release();
  TM_API_END
}

int tm_surrogate_destroy(tm_surrogate* sg) {
  delete sg;
  return TM_OK;
}

int tm_surrogate_gradient_device(tm_surrogate* sg, tm_energy* e, tm_mesh* m, const double* d_points, double* d_grad,
                                 void* stream) {
  TM_API_BEGIN
  if (!sg || !e || !m || !d_points || !d_grad) fail(TM_ERR_ARG, "NULL argument");
  cudaStream_t s = stream ? (cudaStream_t)stream : e->stream;
  surrogate_grad(sg, e, m, d_points, d_grad, s);
  int st = 0;
  TM_CUDA(cudaMemcpyAsync(&st, sg->status.get(), sizeof(int), cudaMemcpyDeviceToHost, s));
  TM_CUDA(cudaStreamSynchronize(s));
  if (st) fail(TM_ERR_TIMEOUT, "tensor-core layer wait timed out (" + std::to_string(st) + ")");
  TM_API_END
}

int tm_surrogate_inputs_device(tm_surrogate* sg, tm_energy* e, tm_mesh* m, const double* d_points, int32_t max_valence,
                               float* d_u, float* d_normals, int32_t* d_nbr, float* d_edge_feat, float* d_dirs,
                               double* d_grad_local, void* stream) {
  TM_API_BEGIN
  if (!sg || !e || !m || !d_points || !d_u || !d_normals || !d_nbr || !d_edge_feat || !d_dirs || !d_grad_local)
    fail(TM_ERR_ARG, "NULL argument");
  if (m->nv != sg->nv) fail(TM_ERR_ARG, "surrogate built for another mesh size");
  if (max_valence < 1 || max_valence > TM_MAXVAL) fail(TM_ERR_ARG, "max_valence out of range");
  cudaStream_t s = stream ? (cudaStream_t)stream : e->stream;
  int nv = m->nv;
  if (nv == 0) return TM_OK;
  std::vector<int> val(nv);
  TM_CUDA(cudaMemcpyAsync(val.data(), m->d_val.get(), sizeof(int) * nv, cudaMemcpyDeviceToHost, s));
  TM_CUDA(cudaStreamSynchronize(s));
  int dmax = *std::max_element(val.begin(), val.end());
  if (dmax > max_valence) fail(TM_ERR_ARG, "a vertex valence exceeds max_valence (" + std::to_string(dmax) + ")");
  energy_eval32_local(e, m, d_points, d_grad_local, s);
  Topo t = m->topo();
  const FaceF* fd = reinterpret_cast<const FaceF*>(e->face.get());
  const EdgeF* ed = reinterpret_cast<const EdgeF*>(e->edge.get());
  const float* rho = reinterpret_cast<const float*>(e->rho.get());
  Split S{e->pos32.get(), e->poslo.get()};
  k_sfeat<<<nblk(nv, 128), 128, 0, s>>>(t, fd, ed, rho, sg->w.get(), d_u, sg->nrm.get(), sg->hb[0].get());
  TM_LAUNCH();
  TM_CUDA(cudaMemcpyAsync(d_normals, sg->nrm.get(), sizeof(float) * 4 * nv, cudaMemcpyDeviceToDevice, s));
  k_export<<<nblk(nv, 128), 128, 0, s>>>(t, S, ed, rho, sg->w.get(), max_valence, d_nbr, d_edge_feat, d_dirs);
  TM_LAUNCH();
  TM_CUDA(cudaStreamSynchronize(s));
  TM_API_END
}

int tm_dense_silu_bf16(const void* d_h, const void* d_m, const void* d_w, const float* d_bias, void* d_out,
                       int64_t rows, void* stream) {
  return tm_dense_silu_bf16_bounded(d_h, d_m, d_w, d_bias, d_out, rows, WAIT_POLLS, stream);
}

int tm_dense_silu_bf16_bounded(const void* d_h, const void* d_m, const void* d_w, const float* d_bias, void* d_out,
                               int64_t rows, int wait_polls, void* stream) {
  TM_API_BEGIN
  if (wait_polls < 0) fail(TM_ERR_ARG, "wait_polls must be >= 0");
  if (!d_h || !d_m || !d_w || !d_bias || !d_out) fail(TM_ERR_ARG, "NULL argument");
  if (rows < 0 || rows > (1LL << 30)) fail(TM_ERR_ARG, "rows out of range");
  cudaStream_t s = (cudaStream_t)stream;
  alignas(64) CUtensorMap mh, mm, mw;
  if (rows == 0) return TM_OK;
  make_map(&mh, d_h, rows, H, BM);
  make_map(&mm, d_m, rows, H, BM);
  make_map(&mw, d_w, H, 2 * H, H);
  DevBuf<int> st;
  st.ensure(1);
  TM_CUDA(cudaMemsetAsync(st.get(), 0, sizeof(int), s));
  dense_launch(mh, mm, mw, d_bias, static_cast<__nv_bfloat16*>(d_out), (int)rows, st.get(), s, wait_polls);
  int hs = 0;
  TM_CUDA(cudaMemcpyAsync(&hs, st.get(), sizeof(int), cudaMemcpyDeviceToHost, s));
  TM_CUDA(cudaStreamSynchronize(s));
  if (hs) fail(TM_ERR_TIMEOUT, "tensor-core layer wait timed out (" + std::to_string(hs) + ")");
  TM_API_END
}


int tm_surrogate_train_create(int64_t n_vertices, int32_t max_valence, const float* weights, int64_t n_weights,
                              tm_strain** out) {
  TM_API_BEGIN
  if (!weights || !out) fail(TM_ERR_ARG, "NULL argument");
  *out = nullptr;
  if (n_vertices < 1 || n_vertices > (1LL << 26)) fail(TM_ERR_ARG, "n_vertices out of range");
  if (max_valence < 1 || max_valence > TM_MAXVAL) fail(TM_ERR_ARG, "max_valence out of range");
  SurW hw{};
  std::vector<__nv_bfloat16> wd;
  parse_blob(weights, n_weights, hw, wd);  // validates the layout
  std::unique_ptr<tm_strain> st(new tm_strain());
  const int nv = (int)n_vertices;
  st->nv = nv;
  st->D = max_valence;
  st->lbar = weights[5];
  st->abar = weights[6];
  st->fscale = weights[7];
  const size_t NH = (size_t)nv * H;
  st->th.ensure(NPARAM);
  st->grad.ensure(NPARAM);
  st->m1.ensure(NPARAM);
  st->m2.ensure(NPARAM);
  st->loss.ensure(1);
  st->wd.ensure((size_t)NR * H * 2 * H);
  st->z.ensure((NR + 1) * NH);
  st->hb.ensure((NR + 1) * NH);
  st->mb.ensure(NR * NH);
  st->dha.ensure(NH);
  st->dhb.ensure(NH);
  st->dm.ensure(NH);
  st->dF.ensure(3 * (size_t)nv);
  st->nb_dense = dense_back_blocks();
  const size_t nb8 = nblk((long)nv * 8, TB), nb16 = nblk((long)nv * 16, TB);
  st->part.ensure(std::max({nb8 * (H * FV + H), nb8 * 130, nb16 * (H * FE + H),
                            (size_t)st->nb_dense * (H * 2 * H + H)}));
  st->lossp.ensure(nb8);
  st->status.ensure(1);
  TM_CUDA(cudaMemcpy(st->th.get(), weights + BLOB_HEADER, sizeof(float) * NPARAM, cudaMemcpyHostToDevice));
  TM_CUDA(cudaMemcpy(st->wd.get(), wd.data(), sizeof(__nv_bfloat16) * wd.size(), cudaMemcpyHostToDevice));
  TM_CUDA(cudaMemset(st->m1.get(), 0, sizeof(float) * NPARAM));
  TM_CUDA(cudaMemset(st->m2.get(), 0, sizeof(float) * NPARAM));
  TM_CUDA(cudaMemset(st->status.get(), 0, sizeof(int)));
  for (int r = 0; r < NR; ++r) {
    make_map(&st->map_h[r], st->hb.get() + r * NH, nv, H, BM);
    make_map(&st->map_m[r], st->mb.get() + r * NH, nv, H, BM);
    make_map(&st->map_w[r], st->wd.get() + (size_t)r * H * 2 * H, H, 2 * H, H);
  }
  *out = st.release();
  TM_API_END
}

int tm_surrogate_train_destroy(tm_strain* st) {
  delete st;
  return TM_OK;
}

int tm_surrogate_train_get_weights(tm_strain* st, float* weights, int64_t n_weights) {
  TM_API_BEGIN
  if (!st || !weights) fail(TM_ERR_ARG, "NULL argument");
  if (n_weights != BLOB_SIZE) fail(TM_ERR_ARG, "weights: expected " + std::to_string(BLOB_SIZE) + " floats");
  const float head[BLOB_HEADER] = {1.0f, (float)FV, (float)FE, (float)H, (float)NR, st->lbar, st->abar, st->fscale};
  std::memcpy(weights, head, sizeof head);
  TM_CUDA(cudaDeviceSynchronize());
  TM_CUDA(cudaMemcpy(weights + BLOB_HEADER, st->th.get(), sizeof(float) * NPARAM, cudaMemcpyDeviceToHost));
  TM_API_END
}

int tm_surrogate_train_grad(tm_strain* st, const float* d_u, const float* d_nrm, const int32_t* d_nbr,
                            const float* d_ef, const float* d_dirs, const float* d_target, int64_t n_vertices,
                            int32_t max_valence, float target_rms, float* d_force, float* d_loss, float* d_grad,
                            void* stream) {
  TM_API_BEGIN
  const TrainInputs in = check_inputs(st, n_vertices, max_valence, d_u, d_nrm, d_nbr, d_ef, d_dirs, d_target);
  if (!(target_rms > 0.0f)) fail(TM_ERR_ARG, "target_rms must be positive");
  cudaStream_t s = (cudaStream_t)stream;
  TM_CUDA(cudaMemsetAsync(st->status.get(), 0, sizeof(int), s));
  const float inv_norm = 1.0f / (3.0f * (float)st->nv * target_rms * target_rms);
  train_pass(st, in, inv_norm, d_grad != nullptr, d_force, s);
  if (d_loss) TM_CUDA(cudaMemcpyAsync(d_loss, st->loss.get(), sizeof(float), cudaMemcpyDeviceToDevice, s));
  if (d_grad)
    TM_CUDA(cudaMemcpyAsync(d_grad, st->grad.get(), sizeof(float) * NPARAM, cudaMemcpyDeviceToDevice, s));
  int hs = 0;
  TM_CUDA(cudaMemcpyAsync(&hs, st->status.get(), sizeof(int), cudaMemcpyDeviceToHost, s));
  TM_CUDA(cudaStreamSynchronize(s));
  if (hs) fail(TM_ERR_TIMEOUT, "tensor-core layer wait timed out (" + std::to_string(hs) + ")");
  TM_API_END
}

int tm_surrogate_train_step(tm_strain* st, const float* d_u, const float* d_nrm, const int32_t* d_nbr,
                            const float* d_ef, const float* d_dirs, const float* d_target, int64_t n_vertices,
                            int32_t max_valence, float target_rms, float lr, float beta1, float beta2, float eps,
                            float* d_loss, void* stream) {
  TM_API_BEGIN
  const TrainInputs in = check_inputs(st, n_vertices, max_valence, d_u, d_nrm, d_nbr, d_ef, d_dirs, d_target);
  if (!(target_rms > 0.0f) || !(lr >= 0.0f) || !(beta1 >= 0.0f && beta1 < 1.0f) ||
      !(beta2 >= 0.0f && beta2 < 1.0f) || !(eps > 0.0f))
    fail(TM_ERR_ARG, "invalid training hyperparameters");
  cudaStream_t s = (cudaStream_t)stream;
  const float inv_norm = 1.0f / (3.0f * (float)st->nv * target_rms * target_rms);
  train_pass(st, in, inv_norm, true, nullptr, s);
  st->step += 1;
  const float c1 = (float)(1.0 / (1.0 - std::pow((double)beta1, (double)st->step)));
  const float c2 = (float)(1.0 / (1.0 - std::pow((double)beta2, (double)st->step)));
  k_t_adam<<<nblk(NPARAM, 256), 256, 0, s>>>(NPARAM, st->th.get(), st->grad.get(), st->m1.get(), st->m2.get(), lr,
                                            beta1, beta2, eps, c1, c2, st->wd.get());
  TM_LAUNCH();
  if (d_loss) TM_CUDA(cudaMemcpyAsync(d_loss, st->loss.get(), sizeof(float), cudaMemcpyDeviceToDevice, s));
  TM_API_END
}

int tm_surrogate_train_status(tm_strain* st) {
  TM_API_BEGIN
  if (!st) fail(TM_ERR_ARG, "NULL argument");
  int hs = 0;
  TM_CUDA(cudaDeviceSynchronize());
  TM_CUDA(cudaMemcpy(&hs, st->status.get(), sizeof(int), cudaMemcpyDeviceToHost));
  if (hs) fail(TM_ERR_TIMEOUT, "tensor-core layer wait timed out (" + std::to_string(hs) + ")");
  TM_API_END
}

}  // extern "C"
