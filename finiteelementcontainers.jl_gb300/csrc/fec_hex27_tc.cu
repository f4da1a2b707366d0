// fec_hex27_tc.cu -- the hex27 element-stiffness contraction on the tensor cores
// (FP32-element variant).
//
// For each element, K_(a,i),(b,k) = sum_q sum_J dN_aJ(q) C_q[(i,J),(b,k)] with
// C_q[(i,J),(b,k)] = sum_L A_q[iJkL] dN_bL(q) (A JxW-scaled).  Stacking i into
// the rows makes it one GEMM per element:
//     D[(i,b,k), a] = sum_{(q,J)} C[(i,b,k),(q,J)] * G[a,(q,J)],  K_(a,i),(b,k) = D[(i,b,k), a]
// with M = 243 rows (two M = 128 tiles), N = 27 (padded to 32) and K = (q,J)
// with J padded to 4, so that one K chunk of 8 is exactly two quadrature points
// (K = 28 x 4 = 112).  The CUDA cores build C chunk by chunk (double buffered,
// shape gradients and tangent entries packed as float4) while the tensor cores
// (tcgen05.mma kind::tf32, FP32 accumulators in tensor memory) consume the
// previous chunk; every operand is a two-term
// TF32 split hi + lo and each product takes hi*hi + lo*hi + hi*lo, which keeps
// the contraction at FP32 accuracy.  The per-point map, constitutive update and
// the residual stay on the CUDA cores, as in the generic kernel.
#include <cstdlib>
#include "../../include/fec_gb300.h"
#include "fec_launch.h"
#include "fec_tc.cuh"

namespace fec {
namespace h27 {

constexpr int A = 27, NQ = 27, ND = 81, KP = 112;         // nodes, points, dofs, padded (q, J) count
constexpr int NCHUNK = KP / 8;                            // 14 chunks of two points
constexpr int NTHR = 256;
constexpr uint32_t SBO_G = (KP / 4) * 128;                // 3584: 8-row groups of the G operand
constexpr uint32_t S_GHI = 0, S_GLO = S_GHI + 4 * SBO_G;  // 32 x 112 tf32 each
constexpr uint32_t S_AOP = S_GLO + 4 * SBO_G;             // 2 buffers x (hi, lo) x 256 x 8 tf32
__host__ __device__ constexpr uint32_t AOP(int buf, int term) { return S_AOP + uint32_t(buf * 2 + term) * 8192; }
constexpr uint32_t S_REFF = S_AOP + 4 * 8192;             // floats: reference tables
constexpr int REF = RefLayout<8>::SIZE;
constexpr uint32_t S_X = S_REFF + ((REF * 4 + 15) & ~15);  // doubles: 81 coordinates
constexpr uint32_t S_U = S_X + ND * 8;                     // floats: 81 displacements
constexpr uint32_t S_XD = S_U + 336;                       // floats: 81 differenced coordinates
constexpr uint32_t S_CONN = S_XD + 336;                    // 27 ints
constexpr uint32_t S_DN4 = (S_CONN + 112 + 15) & ~15u;     // float4 [q][a]: dN_a(q) (x, y, z, 0)
constexpr uint32_t S_P = S_DN4 + NQ * A * 16;              // floats: 27 x 9
constexpr uint32_t S_SCR = S_P + NQ * 9 * 4;               // floats: 27 x 24 (model scratch)
constexpr uint32_t S_A4 = (S_SCR + NQ * 24 * 4 + 15) & ~15u;  // float4 [q][i][J][k]: A_iJk(0..2)
constexpr uint32_t S_BAR = S_A4 + NQ * 27 * 16;            // 2 mbarriers
constexpr uint32_t S_TSLOT = S_BAR + 16;
constexpr uint32_t SMEM = S_TSLOT + 16;
static_assert(S_X % 16 == 0 && S_DN4 % 16 == 0 && S_A4 % 16 == 0 && S_BAR % 8 == 0, "alignment");
static_assert(SMEM <= 113 * 1024, "two CTAs per SM");
constexpr long long WAIT_BUDGET = 2000000000LL;

__device__ __forceinline__ float tf32_hi(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}
// (hi, lo) of four values at (row, k0 .. k0+3) of a K-major tf32 tile with the
// given stride byte offset (k0 a multiple of 4).
__device__ __forceinline__ void store4_split(unsigned char* hi, unsigned char* lo, int row, int k0, uint32_t sbo,
                                             const float* v) {
  float4 h, l;
  h.x = tf32_hi(v[0]); l.x = v[0] - h.x;
  h.y = tf32_hi(v[1]); l.y = v[1] - h.y;
  h.z = tf32_hi(v[2]); l.z = v[2] - h.z;
  h.w = tf32_hi(v[3]); l.w = v[3] - h.w;
  const uint32_t off = uint32_t(row >> 3) * sbo + uint32_t(k0 >> 2) * 128 + uint32_t(row & 7) * 16;
  *reinterpret_cast<float4*>(hi + off) = h;
  *reinterpret_cast<float4*>(lo + off) = l;
}

// kind::tf32, FP32 accumulate, M = 128, N = 32, both K-major
constexpr uint32_t IDESC = (1u << 4) | (2u << 7) | (2u << 10) | (uint32_t(32 >> 3) << 17) | (uint32_t(128 >> 4) << 24);

template <class Model, bool WANT_R, bool WANT_K>
__global__ void __launch_bounds__(NTHR, 2) hex27_tc_kernel(ElemArgs g, int* err) {
  using namespace tc;
  static_assert(WANT_K, "the tensor-core kernel forms K_e");
  constexpr int NS = Model::NS, SCR = Model::SCR;
  static_assert(SCR <= 24, "model scratch");
  extern __shared__ __align__(1024) unsigned char sm[];
  float* s_reff = reinterpret_cast<float*>(sm + S_REFF);
  double* s_x = reinterpret_cast<double*>(sm + S_X);
  float* s_u = reinterpret_cast<float*>(sm + S_U);
  float* s_xd = reinterpret_cast<float*>(sm + S_XD);
  int* s_conn = reinterpret_cast<int*>(sm + S_CONN);
  float4* s_dn4 = reinterpret_cast<float4*>(sm + S_DN4);
  float* s_P = reinterpret_cast<float*>(sm + S_P);
  float* s_scr = reinterpret_cast<float*>(sm + S_SCR);
  float4* s_a4 = reinterpret_cast<float4*>(sm + S_A4);
  uint64_t* bar = reinterpret_cast<uint64_t*>(sm + S_BAR);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t s0 = smem_u32(sm);

  // operand tiles start at zero: padding rows/columns are never written again
  for (int i = tid; i < int(S_REFF / 16); i += NTHR) reinterpret_cast<float4*>(sm)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int i = tid; i < REF; i += NTHR) s_reff[i] = float(g.ref[i]);
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    mbar_fence_init();
  }
  if (warp == 0) tmem_alloc(reinterpret_cast<uint32_t*>(sm + S_TSLOT), 64);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(sm + S_TSLOT);
  uint32_t ph[2] = {0u, 0u};
  bool failed = false;
  // the main waits' budget (settable, fec_set_wait_budget); the drain after a
  // timeout always allows the full WAIT_BUDGET
  const long long budget = g.wait_budget > 0 ? g.wait_budget : WAIT_BUDGET;
  // this thread's row of C: (i, b, k)
  const int row = tid, ri = row / ND, rb = (row % ND) / 3, rk = row % 3;

  for (int64_t e = blockIdx.x; e < g.ne && !failed; e += gridDim.x) {
    // ---- staging ----
    if (tid < A) s_conn[tid] = g.conn[e * A + tid];
    __syncthreads();
    if (tid < ND) {
      const int a = tid / 3, d = tid % 3;
      s_x[tid] = __ldg(&g.coords[int64_t(s_conn[a]) * 3 + d]);
      s_u[tid] = float(__ldg(&g.U[int64_t(s_conn[a]) * 3 + d]));
    }
    __syncthreads();
    if (tid < ND) s_xd[tid] = float(s_x[tid] - s_x[tid % 3]);
    __syncthreads();
    // ---- per point: map, displacement gradient, constitutive update ----
    if (tid < NQ) {
      const int q = tid;
      float dNX[ND];
      const float jxw = map_point_mixed<8>(g.ref, s_reff, q, s_x, s_xd, dNX);
      float gu[3][3];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          float s = 0.f;
#pragma unroll
          for (int a = 0; a < A; ++a) s = fmaf(s_u[a * 3 + i], dNX[a * 3 + j], s);
          gu[i][j] = s;
        }
#pragma unroll
      for (int a = 0; a < A; ++a) s_dn4[q * A + a] = make_float4(dNX[a * 3], dNX[a * 3 + 1], dNX[a * 3 + 2], 0.f);
      const double* so = NS ? g.state_old + (e * NQ + q) * NS : nullptr;
      double* sn = (NS && g.state_new) ? g.state_new + (e * NQ + q) * NS : nullptr;
      Model::point(g.props, gu, jxw, so, sn, s_P + q * 9, s_scr + q * SCR);
    }
    __syncthreads();
    // ---- tangent entries (float4 per (q,i,J,k)), G operand, residual ----
    if (WANT_K && tid < NQ * 3) {
      const int q = tid / 3, i = tid % 3;
      float out[27];
      Model::aentries(s_scr + q * SCR, i, out);
#pragma unroll
      for (int jk = 0; jk < 9; ++jk)
        s_a4[(q * 3 + i) * 9 + jk] = make_float4(out[jk * 3], out[jk * 3 + 1], out[jk * 3 + 2], 0.f);
    }
    if (WANT_K) {
      // G[a, 4q + J] = dN_aJ(q), J = 3 a zero pad
      for (int w = tid; w < A * NQ; w += NTHR) {
        const int a = w / NQ, q = w % NQ;
        const float4 d = s_dn4[q * A + a];
        const float v[4] = {d.x, d.y, d.z, 0.f};
        store4_split(sm + S_GHI, sm + S_GLO, a, 4 * q, SBO_G, v);
      }
    }
    if (WANT_R && tid < ND) {
      const int a = tid / 3, i = tid % 3;
      float R = 0.f;
      for (int q = 0; q < NQ; ++q) {
        const float4 dN = s_dn4[q * A + a];
        const float* P = s_P + q * 9 + i * 3;
        R = fmaf(dN.x, P[0], fmaf(dN.y, P[1], fmaf(dN.z, P[2], R)));
      }
      static_cast<float*>(g.Re)[e * ND + tid] = R;
    }
    __syncthreads();
    // ---- C chunks (two points each), double buffered against the MMAs ----
    for (int c = 0; c < NCHUNK; ++c) {
      const int buf = c & 1;
      if (c >= 2) {
        // the phase flips only when every thread saw it complete, so that after a
        // timeout ph[] still names the phases whose MMAs may be in flight
        const bool ok = mbar_wait(&bar[buf], ph[buf], budget);
        if (__syncthreads_or(!ok)) {
          failed = true;
          break;
        }
        ph[buf] ^= 1u;
      }
      if (row < 3 * ND) {
        float v[8];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int q = 2 * c + h;
          if (q < NQ) {
            const float4 d = s_dn4[q * A + rb];
#pragma unroll
            for (int J = 0; J < 3; ++J) {
              const float4 t = s_a4[((q * 3 + ri) * 3 + J) * 3 + rk];
              v[4 * h + J] = fmaf(t.x, d.x, fmaf(t.y, d.y, t.z * d.z));
            }
            v[4 * h + 3] = 0.f;
          } else {
#pragma unroll
            for (int j = 0; j < 4; ++j) v[4 * h + j] = 0.f;
          }
        }
        store4_split(sm + AOP(buf, 0), sm + AOP(buf, 1), row, 0, 256, v);
        store4_split(sm + AOP(buf, 0), sm + AOP(buf, 1), row, 4, 256, v + 4);
      }
      fence_async_smem();
      tc_fence_before();
      __syncthreads();
      if (tid == 0) {
        tc_fence_after();
        const uint64_t gh = smem_desc(s0 + S_GHI + uint32_t(c) * 256, 128, SBO_G);
        const uint64_t gl = smem_desc(s0 + S_GLO + uint32_t(c) * 256, 128, SBO_G);
#pragma unroll
        for (int t = 0; t < 2; ++t) {
          const uint64_t ah = smem_desc(s0 + AOP(buf, 0) + uint32_t(t) * 4096, 128, 256);
          const uint64_t al = smem_desc(s0 + AOP(buf, 1) + uint32_t(t) * 4096, 128, 256);
          mma_tf32(tmem + 32u * t, ah, gh, IDESC, c > 0);
          mma_tf32(tmem + 32u * t, al, gh, IDESC, 1);
          mma_tf32(tmem + 32u * t, ah, gl, IDESC, 1);
        }
        mma_commit(&bar[buf]);
      }
    }
    if (failed) break;
    // the last two chunks' barriers (chunk 12 on buffer 0, chunk 13 on buffer 1)
    {
      const bool ok0 = mbar_wait(&bar[0], ph[0], budget);
      const bool ok1 = mbar_wait(&bar[1], ph[1], budget);
      if (__syncthreads_or(!(ok0 && ok1))) {
        failed = true;
        break;
      }
      ph[0] ^= 1u;
      ph[1] ^= 1u;
    }
    tc_fence_after();
    // ---- read D back: warp w holds rows 128 (w / 4) + 32 (w % 4) + lane ----
    {
      const int qd = warp & 3, t = warp >> 2;
      const int r = 128 * t + 32 * qd + lane;
      float v[32];
      tmem_ld32(tmem + (uint32_t(32 * qd) << 16) + 32u * t, v);
      if (r < 3 * ND) {
        const int i = r / ND, bk = r % ND;
        float* Ke = static_cast<float*>(g.Ke) + e * (ND * ND) + bk;
#pragma unroll
        for (int a = 0; a < A; ++a) Ke[(a * 3 + i) * ND] = v[a];
      }
    }
    tc_fence_before();
    __syncthreads();
  }
  if (failed) {
    // one more bounded wait on each barrier's pending phase (a phase that already
    // completed returns at once), so that no MMA is left writing TMEM below
    if (tid == 0) atomicExch(err, 1);
    mbar_wait(&bar[0], ph[0], WAIT_BUDGET);
    mbar_wait(&bar[1], ph[1], WAIT_BUDGET);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, 64);
  }
}

int sm_count() {
  static int count[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 148;
  if (!count[dev]) cudaDeviceGetAttribute(&count[dev], cudaDevAttrMultiProcessorCount, dev);
  return count[dev] > 0 ? count[dev] : 148;
}

template <class Model, bool R, bool K>
cudaError_t go(const ElemArgs& a, int* err, cudaStream_t s) {
  cudaError_t e = ensure_smem<hex27_tc_kernel<Model, R, K>>(SMEM);
  if (e != cudaSuccess) return e;
  const int64_t cap = int64_t(2) * sm_count();
  const unsigned grid = unsigned(a.ne < cap ? a.ne : cap);
  hex27_tc_kernel<Model, R, K><<<grid, NTHR, SMEM, s>>>(a, err);
  return cudaGetLastError();
}

template <class Model>
cudaError_t launch(bool want_r, bool want_k, const ElemArgs& a, int* err, cudaStream_t s, int* launches) {
  if (!want_k) return cudaErrorNotSupported;  // residual only: no contraction, the generic kernel serves it
  if (a.ne <= 0) return cudaSuccess;
  ++*launches;
  if (want_r) return go<Model, true, true>(a, err, s);
  return go<Model, false, true>(a, err, s);
}

}  // namespace h27

bool hex27_on_cuda_cores() {
  const char* v = std::getenv("FEC_HEX27_ON_CUDA_CORES");
  return v && v[0] == '1';
}

namespace {
// set by an element kernel whose bounded wait gave up: a hex27 tensor-core
// kernel waiting on its MMAs, or a hex8 kernel waiting on its bulk table copies
__device__ int g_wait_error = 0;
}  // namespace

cudaError_t wait_error_flag(int** flag) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_wait_error);
  *flag = static_cast<int*>(p);
  return e;
}

cudaError_t launch_hex27_tc(int physics, bool want_r, bool want_k, const ElemArgs& a, cudaStream_t s,
                            int* launches) {
  int* err = a.wait_err;
  if (!err) {
    const cudaError_t e = wait_error_flag(&err);
    if (e != cudaSuccess) return e;
  }
  if (physics == 2) return h27::launch<NeoHookean>(want_r, want_k, a, err, s, launches);
  if (physics == 3) return h27::launch<J2>(want_r, want_k, a, err, s, launches);
  return cudaErrorNotSupported;
}

}  // namespace fec

extern "C" int fec_tensor_core_status(int reset) {
  int* flag = nullptr;
  if (fec::wait_error_flag(&flag) != cudaSuccess) return FEC_ERR_CUDA;
  int h = 0;
  if (cudaMemcpy(&h, flag, sizeof h, cudaMemcpyDeviceToHost) != cudaSuccess) return FEC_ERR_CUDA;
  if (reset && cudaMemset(flag, 0, sizeof h) != cudaSuccess) return FEC_ERR_CUDA;
  return h ? FEC_ERR_DEVICE : FEC_OK;
}
