// fec_class_tc.cu -- FP32-element tet10 / hex27 element stiffness on the tensor
// cores for element blocks made of a few translation classes: element e is a
// translate of element e mod P (P <= 8).  The structured boxes of the
// mixed-element workloads are such blocks: hex27 boxes one class, tet10 boxes
// the six Kuhn tets of a cube.
//
// The tangent of element e is (src/Formulations.jl:462-576)
//     K_(a,i),(b,k) = sum_q sum_(J,L) dNX_qaJ * JxW A_q,iJkL * dNX_qbL .
// Within a class dNX_q and JxW_q are the same for every element, so with
// r = (q, J, L) (9 NQ values) and the node pair n = (a, b), a <= b,
//     D[(e, i, k), n] = sum_r A_e[(e, i, k), r] * W[n, r],   W[n, r] = dNX_qaJ dNX_qbL,
// one GEMM per tile of 12 elements of one class against the class's constant
// W: M = 128 rows (e, i, k) (three elements per 32-row quarter, lanes 27-31 of
// each quarter padding), N = the pairs (55 -> 64 for tet10, 378 -> 384 for
// hex27), K = 9 NQ in steps of 8.  tcgen05.mma kind::tf32 with two-term splits
// of both operands (hi*hi + lo*hi + hi*lo: FP32 accuracy) accumulates in FP32 in
// tensor memory.  The other half of K_e follows from K = K^T (A_iJkL = A_kLiJ).
//
// Per tile: the elements' connectivity and displacement differences u_a - u_0
// (FP64 differences, then FP32), the per-point constitutive update from the
// class's constant gradients (no isoparametric map) and the point's 45 unique
// JxW A entries, the residual, then the K loop: every thread builds its share of
// the A slice of step s (entries looked up, split into tf32 hi/lo) while the MMAs
// of step s-1 run; one thread streams the class's W image of step s + NWB - 2
// from global memory (L2) with a bulk copy and issues the MMAs of step s.  The
// epilogue reads the accumulator rows back and writes the symmetric half of K_e
// as it comes out of tensor memory (the KE_PAIRS workspace layout: pair n, then
// the nine (i, k); the node gather reads the other half transposed).  Every
// mbarrier wait is bounded; a wait that gives up sets the flag
// fec_tensor_core_status reads, drains the operations in flight and ends the
// kernel.
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "fec_kernels.cuh"
#include "fec_launch.h"
#include "fec_mech_hex27.cuh"
#include "fec_tc.cuh"

namespace fec {
namespace ctc {

template <int ET>
struct Shape;
template <>
struct Shape<7> {  // TETRA10, 4-point rule
  static constexpr int A = 10, NQ = 4, NPAD = 64, NPART = 64, MINB = 2, TMEM_COLS = 64, NWB = 3;
};
template <>
struct Shape<8> {  // HEX27, 27-point rule
  static constexpr int A = 27, NQ = 27, NPAD = 384, NPART = 192, MINB = 1, TMEM_COLS = 512, NWB = 4;
};

constexpr int EPT = 12;  // elements per tile
constexpr int NTHR = 256;
constexpr int HEADER = 64;
constexpr long long WAIT_BUDGET = 2000000000LL;

template <int ET>
struct L {
  using S = Shape<ET>;
  static constexpr int A = S::A, NQ = S::NQ, NDOF = 3 * A, NP = A * (A + 1) / 2, KR = 9 * NQ;
  static constexpr int KSTEPS = (KR + 7) / 8, NPAD = S::NPAD, NPART = S::NPART, NPARTS = NPAD / NPART;
  static constexpr int W_TERM = NPAD * 32;    // bytes of one tf32 term of one K step (NPAD rows x 8)
  static constexpr int W_STEP = 2 * W_TERM;   // hi image, then lo image
  static constexpr int G_FLOATS = NQ * A * 3 + NQ;
  static constexpr int G_BYTES = (G_FLOATS * 4 + 15) / 16 * 16;
  static constexpr int CLASS_BYTES = KSTEPS * W_STEP + G_BYTES;
  static_assert(NP <= NPAD && NPAD % NPART == 0 && NPART % 16 == 0 && NPART <= 256, "N");
  static_assert(W_STEP % 16 == 0 && CLASS_BYTES % 16 == 0, "alignment");
};

// shared-memory layout (bytes).  NWB W buffers: the
// image of step s + NWB - 2 is requested at step s (once the MMAs of step s - 2,
// the last reader of its buffer, completed), NWB - 2 steps ahead of its use.
template <int ET, class Model>
struct Smem {
  using G = L<ET>;
  static constexpr int NWB = Shape<ET>::NWB;
  static constexpr int W = 0;                                   // NWB x W_STEP
  static constexpr int AOP = W + NWB * G::W_STEP;               // 2 buffers x (hi, lo) x 4096
  static constexpr int ENT = AOP + 2 * 8192;                    // floats [EPT][NQ][45]: JxW A, unique entries
  static constexpr int P = ENT + EPT * G::NQ * 45 * 4;          // floats [EPT][NQ][9]: JxW P
  static constexpr int GR = (P + EPT * G::NQ * 9 * 4 + 15) / 16 * 16;  // class gradients + JxW
  static constexpr int U = GR + G::G_BYTES;                      // floats [EPT][A][3]
  static constexpr int CONN = U + EPT * G::A * 3 * 4;            // ints [EPT][A]
  static constexpr int BAR = (CONN + EPT * G::A * 4 + 15) / 16 * 16;  // NWB W barriers, 2 MMA barriers
  static constexpr int TSLOT = BAR + (NWB + 2) * 8;
  static constexpr int BYTES = TSLOT + 16;
  static_assert(BYTES <= 232448, "shared memory");
};

__device__ __forceinline__ float tf32_hi(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}
// (hi, lo) of four values at (row, k0 .. k0+3), k0 in {0, 4}, of a 128 x 8 tf32 tile
__device__ __forceinline__ void store4_split(unsigned char* hi, unsigned char* lo, int row, int k0, const float* v) {
  float4 h, l;
  h.x = tf32_hi(v[0]); l.x = v[0] - h.x;
  h.y = tf32_hi(v[1]); l.y = v[1] - h.y;
  h.z = tf32_hi(v[2]); l.z = v[2] - h.z;
  h.w = tf32_hi(v[3]); l.w = v[3] - h.w;
  const uint32_t off = uint32_t(row >> 3) * 256u + uint32_t(k0 >> 2) * 128u + uint32_t(row & 7) * 16u;
  *reinterpret_cast<float4*>(hi + off) = h;
  *reinterpret_cast<float4*>(lo + off) = l;
}

// kind::tf32, FP32 accumulate, both operands K-major, M = 128
__host__ __device__ constexpr uint32_t idesc_tf32(int N) {
  return (1u << 4) | (2u << 7) | (2u << 10) | (uint32_t(N >> 3) << 17) | (uint32_t(128 >> 4) << 24);
}

// element of tile (class c, tile u within the class), slot el
__device__ __forceinline__ int64_t tile_elem(int c, int64_t u, int el, int P) {
  return int64_t(c) + int64_t(P) * (u * EPT + el);
}

template <int ET, class Model, bool WANT_R, bool WANT_K>
__global__ void __launch_bounds__(NTHR, Shape<ET>::MINB) class_tc_kernel(ElemArgs g, int* err) {
  using namespace tc;
  using G = L<ET>;
  using Sm = Smem<ET, Model>;
  constexpr int A = G::A, NQ = G::NQ, NDOF = G::NDOF, SCR = Model::SCR, NS = Model::NS;
  extern __shared__ __align__(1024) unsigned char sm[];
  const unsigned char* tab = static_cast<const unsigned char*>(g.affine);
  const int P = reinterpret_cast<const int*>(tab)[0], off32 = reinterpret_cast<const int*>(tab)[1];
  float* s_ent = reinterpret_cast<float*>(sm + Sm::ENT);
  float* s_P = reinterpret_cast<float*>(sm + Sm::P);
  float* s_g = reinterpret_cast<float*>(sm + Sm::GR);  // dNX [q][a][3], then JxW [q]
  float* s_u = reinterpret_cast<float*>(sm + Sm::U);
  int* s_conn = reinterpret_cast<int*>(sm + Sm::CONN);
  constexpr int NWB = Sm::NWB;
  uint64_t* wbar = reinterpret_cast<uint64_t*>(sm + Sm::BAR);
  uint64_t* mbar = wbar + NWB;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t s0 = smem_u32(sm);

  // ---- setup: A buffers zero (padding rows are never written) ----
  for (int i = tid; i < 2 * 8192 / 16; i += NTHR)
    reinterpret_cast<float4*>(sm + Sm::AOP)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
  if (tid == 0) {
    for (int i = 0; i < NWB; ++i) mbar_init(&wbar[i], 1);
    mbar_init(&mbar[0], 1);
    mbar_init(&mbar[1], 1);
    mbar_fence_init();
  }
  if (warp == 0) tmem_alloc(reinterpret_cast<uint32_t*>(sm + Sm::TSLOT), Shape<ET>::TMEM_COLS);
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(sm + Sm::TSLOT);
  const long long budget = g.wait_budget > 0 ? g.wait_budget : WAIT_BUDGET;
  uint32_t wph[NWB], mph[2] = {0u, 0u};
  bool wpend[NWB];  // thread 0: a W copy in flight per buffer
  for (int i = 0; i < NWB; ++i) {
    wph[i] = 0u;
    wpend[i] = false;
  }
  bool failed = false;

  // tiles: class-major, ceil(n_c / EPT) per class, n_c = elements of class c
  int64_t ntiles = 0;
  for (int c = 0; c < P; ++c) ntiles += ((g.ne - c + P - 1) / P + EPT - 1) / EPT;
  int cur = -1;
  for (int64_t t = blockIdx.x; t < ntiles && !failed; t += gridDim.x) {
    int c = 0;
    int64_t u = t;
    for (;;) {
      const int64_t nt = ((g.ne - c + P - 1) / P + EPT - 1) / EPT;
      if (u < nt) break;
      u -= nt;
      ++c;
    }
    const unsigned char* ctab = tab + off32 + size_t(c) * G::CLASS_BYTES;
    // W steps 0 .. NWB-1 of this tile (every W buffer is free: the previous tile's MMAs completed)
    if (WANT_K && tid == 0) {
      for (int j = 0; j < NWB && j < G::KSTEPS; ++j) {
        mbar_expect_tx(&wbar[j], uint32_t(G::W_STEP));
        bulk_g2s(sm + Sm::W + j * G::W_STEP, ctab + size_t(j) * G::W_STEP, uint32_t(G::W_STEP), &wbar[j]);
        wpend[j] = true;
      }
    }
    if (c != cur) {
      const float* gsrc = reinterpret_cast<const float*>(ctab + size_t(G::KSTEPS) * G::W_STEP);
      for (int i = tid; i < G::G_FLOATS; i += NTHR) s_g[i] = __ldg(gsrc + i);
      cur = c;
    }
    for (int i = tid; i < EPT * A; i += NTHR) {
      const int el = i / A, a = i - el * A;
      const int64_t e = tile_elem(c, u, el, P);
      s_conn[i] = e < g.ne ? g.conn[e * A + a] : -1;
    }
    __syncthreads();
    // displacement differences u_a - u_0 (FP64, then FP32)
    for (int i = tid; i < EPT * A * 3; i += NTHR) {
      const int el = i / (A * 3), r = i - el * A * 3, a = r / 3, d = r - a * 3;
      const int n = s_conn[el * A + a], n0 = s_conn[el * A];
      s_u[i] = n >= 0 ? float(__ldg(&g.U[int64_t(n) * 3 + d]) - __ldg(&g.U[int64_t(n0) * 3 + d])) : 0.f;
    }
    __syncthreads();
    // ---- per point: displacement gradient and constitutive update ----
    for (int p = tid; p < EPT * NQ; p += NTHR) {
      const int el = p / NQ, q = p - el * NQ;
      const int64_t e = tile_elem(c, u, el, P);
      float* Pq = s_P + p * 9;
      float* ent = s_ent + p * 45;
      if (e < g.ne) {
        const float* dnx = s_g + q * A * 3;
        const float* ue = s_u + el * A * 3;
        float gu[3][3];
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
          for (int j = 0; j < 3; ++j) gu[i][j] = 0.f;
        for (int a = 1; a < A; ++a) {
          const float u0 = ue[a * 3], u1 = ue[a * 3 + 1], u2 = ue[a * 3 + 2];
#pragma unroll
          for (int j = 0; j < 3; ++j) {
            const float dj = dnx[a * 3 + j];
            gu[0][j] = fmaf(u0, dj, gu[0][j]);
            gu[1][j] = fmaf(u1, dj, gu[1][j]);
            gu[2][j] = fmaf(u2, dj, gu[2][j]);
          }
        }
        const double* so = NS ? g.state_old + (e * NQ + q) * NS : nullptr;
        double* sn = (NS && g.state_new) ? g.state_new + (e * NQ + q) * NS : nullptr;
        float scr[SCR];
        Model::point(g.props, gu, s_g[NQ * A * 3 + q], so, sn, Pq, scr);
        // unique entries w = (r1, r2), r1 = 3i + J <= r2 = 3k + L, in row order
#pragma unroll
        for (int r1 = 0, w = 0; r1 < 9; ++r1)
#pragma unroll
          for (int r2 = r1; r2 < 9; ++r2, ++w) ent[w] = Model::aentry(scr, r1 / 3, r1 % 3, r2 / 3, r2 % 3);
      } else {
        for (int m = 0; m < 9; ++m) Pq[m] = 0.f;
        for (int m = 0; m < 45; ++m) ent[m] = 0.f;
      }
    }
    __syncthreads();
    if (WANT_R) {
      for (int i = tid; i < EPT * NDOF; i += NTHR) {
        const int el = i / NDOF, r = i - el * NDOF, a = r / 3, ii = r - a * 3;
        const int64_t e = tile_elem(c, u, el, P);
        if (e >= g.ne) continue;
        float R = 0.f;
        for (int q = 0; q < NQ; ++q) {
          const float* dn = s_g + (q * A + a) * 3;
          const float* Pq = s_P + (el * NQ + q) * 9 + ii * 3;
          R = fmaf(dn[0], Pq[0], fmaf(dn[1], Pq[1], fmaf(dn[2], Pq[2], R)));
        }
        static_cast<float*>(g.Re)[e * NDOF + r] = R;
      }
    }
    if (!WANT_K) {  // residual only: the next tile may reuse the point data
      __syncthreads();
      continue;
    }
    // ---- K loop: A slices double buffered against the MMAs, W streamed ----
    const int row = tid >> 1, half = tid & 1;
    const int rq = row & 31, rel = 3 * (row >> 5) + rq / 9, rik = rq % 9;
    for (int s = 0; s < G::KSTEPS; ++s) {
      const int buf = s & 1;
      if (s >= 2) {  // MMAs of step s-2 read A[buf] and W[(s-2) % NWB]
        const bool ok = mbar_wait(&mbar[buf], mph[buf], budget);
        if (__syncthreads_or(!ok)) {
          failed = true;
          break;
        }
        mph[buf] ^= 1u;
      }
      if (tid == 0 && s >= 2 && s + NWB - 2 < G::KSTEPS) {
        const int j = s + NWB - 2, wb = j % NWB;
        mbar_expect_tx(&wbar[wb], uint32_t(G::W_STEP));
        bulk_g2s(sm + Sm::W + wb * G::W_STEP, ctab + size_t(j) * G::W_STEP, uint32_t(G::W_STEP), &wbar[wb]);
        wpend[wb] = true;
      }
      if (rq < 27) {
        const int i = rik / 3, k = rik - i * 3;
        float v[4];
#pragma unroll
        for (int cc = 0; cc < 4; ++cc) {
          const int r = 8 * s + 4 * half + cc;
          v[cc] = 0.f;
          if (r < G::KR) {
            const int q = r / 9, JL = r - q * 9;
            const int ra = 3 * i + JL / 3, rb = 3 * k + JL % 3;  // A_iJkL = A_kLiJ
            const int r1 = ra < rb ? ra : rb, r2 = ra < rb ? rb : ra;
            v[cc] = s_ent[(rel * NQ + q) * 45 + r1 * 9 - (r1 * (r1 - 1)) / 2 + (r2 - r1)];
          }
        }
        store4_split(sm + Sm::AOP + buf * 8192, sm + Sm::AOP + buf * 8192 + 4096, row, 4 * half, v);
      }
      fence_async_smem();
      tc_fence_before();
      __syncthreads();
      if (tid == 0) {
        const int wb = s % NWB;
        bool ok = mbar_wait(&wbar[wb], wph[wb], budget);
        if (!ok) {  // report, then wait the copy out so that it does not land later
          atomicExch(err, 1);
          mbar_wait(&wbar[wb], wph[wb], WAIT_BUDGET);
        }
        wph[wb] ^= 1u;
        wpend[wb] = false;
        tc_fence_after();
        const uint32_t wbase = s0 + uint32_t(Sm::W + wb * G::W_STEP);
        const uint32_t abase = s0 + uint32_t(Sm::AOP + buf * 8192);
        const uint64_t ah = smem_desc(abase, 128, 256), al = smem_desc(abase + 4096, 128, 256);
#pragma unroll
        for (int pp = 0; pp < G::NPARTS; ++pp) {
          const uint32_t boff = uint32_t(pp * (G::NPART / 8) * 256);
          const uint64_t bh = smem_desc(wbase + boff, 128, 256), bl = smem_desc(wbase + G::W_TERM + boff, 128, 256);
          const uint32_t d = tmem + uint32_t(pp * G::NPART);
          mma_tf32(d, ah, bh, idesc_tf32(G::NPART), s > 0);
          mma_tf32(d, al, bh, idesc_tf32(G::NPART), 1);
          mma_tf32(d, ah, bl, idesc_tf32(G::NPART), 1);
        }
        mma_commit(&mbar[buf]);
      }
    }
    if (failed) break;
    {  // the last two steps' MMAs (one step when KSTEPS == 1)
      bool ok = true;
      for (int s = G::KSTEPS >= 2 ? G::KSTEPS - 2 : 0; s < G::KSTEPS; ++s) {
        ok = mbar_wait(&mbar[s & 1], mph[s & 1], budget) && ok;
      }
      if (__syncthreads_or(!ok)) {
        failed = true;
        break;
      }
      for (int s = G::KSTEPS >= 2 ? G::KSTEPS - 2 : 0; s < G::KSTEPS; ++s) mph[s & 1] ^= 1u;
    }
    tc_fence_after();
    // ---- epilogue: accumulator rows -> the symmetric half of K_e (KE_PAIRS) ----
    {
      const int qd = warp & 3, ch = warp >> 2;
      const int j = lane / 9, ik = lane - 9 * j;
      const int64_t e = tile_elem(c, u, 3 * qd + j, P);
      const bool mine = lane < 27 && e < g.ne;
      float* dst = static_cast<float*>(g.Ke) + e * (G::NP * 9) + ik;
      constexpr int HALF = G::NPAD / 2;
      for (int c0 = ch * HALF; c0 < (ch + 1) * HALF; c0 += 32) {
        float v[32];
        tmem_ld32(tmem + (uint32_t(32 * qd) << 16) + uint32_t(c0), v);
        if (mine) {
#pragma unroll
          for (int cc = 0; cc < 32; ++cc)
            if (c0 + cc < G::NP) dst[(c0 + cc) * 9] = v[cc];
        }
      }
    }
    tc_fence_before();
    __syncthreads();
  }
  if (failed) {
    // one more bounded wait on each barrier's pending phase (a phase that already
    // completed returns at once), so that no MMA or copy is left in flight
    if (tid == 0) {
      atomicExch(err, 1);
      for (int i = 0; i < NWB; ++i)
        if (wpend[i]) mbar_wait(&wbar[i], wph[i], WAIT_BUDGET);
    }
    mbar_wait(&mbar[0], mph[0], WAIT_BUDGET);
    mbar_wait(&mbar[1], mph[1], WAIT_BUDGET);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, Shape<ET>::TMEM_COLS);
  }
}

template <int ET, class Model, bool R, bool K>
cudaError_t go(const ElemArgs& a, int* err, cudaStream_t s) {
  constexpr int smem = Smem<ET, Model>::BYTES;
  cudaError_t e = ensure_smem<class_tc_kernel<ET, Model, R, K>>(size_t(smem));
  if (e != cudaSuccess) return e;
  // the class count P <= 8 is read on the device; its tiles number at most ceil(ne / EPT) + P
  const int64_t tiles = (a.ne + EPT - 1) / EPT + 8;
  const int64_t cap = int64_t(Shape<ET>::MINB) * num_sms();
  const unsigned grid = unsigned(tiles < cap ? tiles : cap);
  class_tc_kernel<ET, Model, R, K><<<grid, NTHR, smem, s>>>(a, err);
  return cudaGetLastError();
}

template <int ET, class Model>
cudaError_t launch(bool want_r, bool want_k, const ElemArgs& a, int* err, cudaStream_t s, int* launches) {
  if (a.ne <= 0 || (!want_r && !want_k)) return cudaSuccess;
  ++*launches;
  if (!want_k) return go<ET, Model, true, false>(a, err, s);
  return want_r ? go<ET, Model, true, true>(a, err, s) : go<ET, Model, false, true>(a, err, s);
}

// ---------------------------------------------------------------------------
// FP64 tet10 blocks of translation classes: the same GEMM with FP64 accuracy from
// BF16 tensor cores, by exact digit slicing of both operands (the scheme of the
// FP64 hex8 kernel, fec_hex8_affine_tc.cu: the Ozaki scheme, Ozaki, Ogita, Oishi
// and Rump, Numer. Algorithms 59 (2012) 95-118, restated for BF16 digits).  Each
// A row (element e, scaled by 2^(7 - tau_e) above its largest tangent entry) and
// each W row (pair n, 2^(7 - sigma_n)) is seven signed 8-bit digits, exact in
// BF16; the digit products of level L = s + t (s + t <= 6) accumulate exactly in
// their own FP32 accumulator (36 reduction terms: below 2^23), seven levels x 64
// pairs = 448 TMEM columns; the epilogue sums the levels in double-float and
// scales by 2^(tau_e + sigma_n - 14).  Per tile of 12 elements: the FP64 point
// phase (displacement gradient from absolute displacements and the class's FP64
// gradients, constitutive update, the double-float scratch, the 45 unique tangent
// entries in double-float, the element scale), the residual in double-float, the
// A digit slices of the three K steps (K = 36 padded to 48), 30 MMAs (10 groups of
// digit pairs per K step, consecutive W slices as one N = 64..256 operand), the
// epilogue into the KE_PAIRS workspace (double-float pairs).
// ---------------------------------------------------------------------------
namespace x64 {
constexpr int A = 10, NQ = 4, NDOF = 30, NP = 55, NPAD = 64, KR = 36, KS = 3, EPT = 12, NPT = EPT * NQ;
constexpr int ND = 7, NLEV = 7;
constexpr int A_SLICE = 128 * 16 * 2, A_STEP = ND * A_SLICE;  // one digit of one K step; the seven digits
constexpr int W_SLICE = NPAD * 16 * 2, W_STEP = ND * W_SLICE, W_BYTES = KS * W_STEP;
// class section: W digit images [KS][ND][NPAD x 16], sigma int[NPAD], dNX double [NQ][A][3], JxW double [NQ]
constexpr int C_W = 0, C_SIG = W_BYTES, C_G = C_SIG + NPAD * 4, C_JXW = C_G + NQ * A * 3 * 8;
constexpr int C_BYTES = (C_JXW + NQ * 8 + 15) / 16 * 16;
static_assert(W_BYTES % 16 == 0 && C_G % 8 == 0, "class section layout");
// shared memory
constexpr int S_A = 0, S_W = S_A + KS * A_STEP, S_ENT = S_W + W_BYTES;  // float2 [NPT][45]
constexpr int S_P2 = S_ENT + NPT * 45 * 8;                             // float2 [NPT][9]
constexpr int S_G = S_P2 + NPT * 9 * 8;                                // double [NQ][A][3]
constexpr int S_G2 = S_G + NQ * A * 3 * 8;                             // float2 [NQ][A][3]
constexpr int S_JXW = S_G2 + NQ * A * 3 * 8;                           // double [NQ]
constexpr int S_SIG = S_JXW + NQ * 8;                                  // int [NPAD]
constexpr int S_U = S_SIG + NPAD * 4;                                  // double [EPT][A][3]
constexpr int S_CONN = S_U + EPT * A * 3 * 8;                          // int [EPT][A]
constexpr int S_SCR = S_CONN + EPT * A * 4;                            // float2 [NPT][SCR2_MAX]: split scratch
constexpr int SCR2_MAX = 24;
constexpr int S_BND = S_SCR + NPT * SCR2_MAX * 8;                      // float [NPT]
constexpr int S_TAU = S_BND + NPT * 4;                                 // int [16]
constexpr int S_BAR = (S_TAU + 16 * 4 + 15) / 16 * 16;                 // W, MMA barriers
constexpr int S_TSLOT = S_BAR + 16;
constexpr int SMEM = S_TSLOT + 16;
static_assert(SMEM <= 232448, "shared memory");
constexpr int NGROUP = 10;
// (A slice t, first W slice s0, W slices ns): every digit pair s + t <= 6 once; the
// t = 0 groups write each level first
__device__ __constant__ int8_t kGroups[NGROUP][3] = {{0, 0, 4}, {0, 4, 3}, {1, 0, 4}, {1, 4, 2}, {2, 0, 4},
                                                      {2, 4, 1}, {3, 0, 4}, {4, 0, 3}, {5, 0, 2}, {6, 0, 1}};

// byte offset of (row, col) in a K-major BF16 operand tile with K = 16
__host__ __device__ __forceinline__ uint32_t op16(int row, int col) {
  return uint32_t(row >> 3) * 256u + uint32_t(col >> 3) * 128u + uint32_t(row & 7) * 16u + uint32_t(col & 7) * 2u;
}
// 2^k as a float for k in [-126, 127]
__device__ __forceinline__ float pow2f(int k) { return __uint_as_float(uint32_t(k + 127) << 23); }
// Seven 4-column loads (the seven levels of four pairs, levels 64 columns apart) under one wait
__device__ __forceinline__ void tmem_ld4x7(uint32_t taddr, float (*v)[4]) {
  uint32_t r[28];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0, %1, %2, %3}, [%28];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%4, %5, %6, %7}, [%29];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%8, %9, %10, %11}, [%30];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%12, %13, %14, %15}, [%31];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%16, %17, %18, %19}, [%32];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%20, %21, %22, %23}, [%33];\n\t"
      "tcgen05.ld.sync.aligned.32x32b.x4.b32 {%24, %25, %26, %27}, [%34];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27])
      : "r"(taddr), "r"(taddr + 64u), "r"(taddr + 128u), "r"(taddr + 192u), "r"(taddr + 256u), "r"(taddr + 320u),
        "r"(taddr + 384u)
      : "memory");
#pragma unroll
  for (int L = 0; L < NLEV; ++L)
#pragma unroll
    for (int j = 0; j < 4; ++j) v[L][j] = __uint_as_float(r[L * 4 + j]);
}

template <class Model, bool WANT_R, bool WANT_K>
__global__ void __launch_bounds__(NTHR, 1) class_tc64_kernel(ElemArgs g, int* err) {
  using namespace tc;
  constexpr int NS = Model::NS;
  extern __shared__ __align__(1024) unsigned char sm[];
  const unsigned char* tab = static_cast<const unsigned char*>(g.affine);
  const int P = reinterpret_cast<const int*>(tab)[0], off64 = reinterpret_cast<const int*>(tab)[2];
  float2* s_ent = reinterpret_cast<float2*>(sm + S_ENT);
  float2* s_P2 = reinterpret_cast<float2*>(sm + S_P2);
  double* s_g = reinterpret_cast<double*>(sm + S_G);
  float2* s_g2 = reinterpret_cast<float2*>(sm + S_G2);
  double* s_jxw = reinterpret_cast<double*>(sm + S_JXW);
  int* s_sig = reinterpret_cast<int*>(sm + S_SIG);
  double* s_u = reinterpret_cast<double*>(sm + S_U);
  int* s_conn = reinterpret_cast<int*>(sm + S_CONN);
  float* s_bnd = reinterpret_cast<float*>(sm + S_BND);
  int* s_tau = reinterpret_cast<int*>(sm + S_TAU);
  float2* s_scr2 = reinterpret_cast<float2*>(sm + S_SCR);
  static_assert(Model::SCR2 <= SCR2_MAX, "scratch");
  uint64_t* wbar = reinterpret_cast<uint64_t*>(sm + S_BAR);
  uint64_t* mbar = wbar + 1;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t s0 = smem_u32(sm);

  // ---- setup: A slices zero (padding rows are never written) ----
  for (int i = tid; i < KS * A_STEP / 16; i += NTHR)
    reinterpret_cast<uint4*>(sm + S_A)[i] = make_uint4(0u, 0u, 0u, 0u);
  if (tid == 0) {
    mbar_init(wbar, 1);
    mbar_init(mbar, 1);
    mbar_fence_init();
  }
  if (warp == 0) tmem_alloc(reinterpret_cast<uint32_t*>(sm + S_TSLOT), 512);
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *reinterpret_cast<volatile uint32_t*>(sm + S_TSLOT);
  const long long budget = g.wait_budget > 0 ? g.wait_budget : WAIT_BUDGET;
  uint32_t wph = 0u, mph = 0u;
  bool wpend = false, failed = false;

  int64_t ntiles = 0;
  for (int c = 0; c < P; ++c) ntiles += ((g.ne - c + P - 1) / P + EPT - 1) / EPT;
  int cur = -1;
  for (int64_t t = blockIdx.x; t < ntiles && !failed; t += gridDim.x) {
    int c = 0;
    int64_t u = t;
    for (;;) {
      const int64_t nt = ((g.ne - c + P - 1) / P + EPT - 1) / EPT;
      if (u < nt) break;
      u -= nt;
      ++c;
    }
    const unsigned char* ctab = tab + off64 + size_t(c) * C_BYTES;
    if (c != cur) {
      // the class's W digits (the previous tile's MMAs completed) and gradients
      if (WANT_K && tid == 0) {
        mbar_expect_tx(wbar, uint32_t(W_BYTES));
        bulk_g2s(sm + S_W, ctab + C_W, uint32_t(W_BYTES), wbar);
        wpend = true;
      }
      for (int i = tid; i < NQ * A * 3; i += NTHR) {
        const double v = __ldg(reinterpret_cast<const double*>(ctab + C_G) + i);
        s_g[i] = v;
        s_g2[i] = df64_split(v);
      }
      if (tid < NQ) s_jxw[tid] = __ldg(reinterpret_cast<const double*>(ctab + C_JXW) + tid);
      if (tid < NPAD) s_sig[tid] = __ldg(reinterpret_cast<const int*>(ctab + C_SIG) + tid);
      cur = c;
    }
    for (int i = tid; i < EPT * A; i += NTHR) {
      const int el = i / A, a = i - el * A;
      const int64_t e = tile_elem(c, u, el, P);
      s_conn[i] = e < g.ne ? g.conn[e * A + a] : -1;
    }
    __syncthreads();
    for (int i = tid; i < EPT * A * 3; i += NTHR) {
      const int el = i / (A * 3), r = i - el * A * 3, a = r / 3, d = r - a * 3;
      const int n = s_conn[el * A + a];
      s_u[i] = n >= 0 ? __ldg(&g.U[int64_t(n) * 3 + d]) : 0.0;
    }
    __syncthreads();
    // ---- per point (FP64): displacement gradient, constitutive update ----
    if (tid < NPT) {
      const int el = tid / NQ, q = tid - el * NQ;
      const int64_t e = tile_elem(c, u, el, P);
      float2* P2 = s_P2 + tid * 9;
      float2* scr2 = s_scr2 + tid * SCR2_MAX;
      float bnd = 0.f;
      if (e < g.ne) {
        const double* gq = s_g + q * A * 3;
        const double* ue = s_u + el * A * 3;
        double gu[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        for (int a = 0; a < A; ++a)
#pragma unroll
          for (int j = 0; j < 3; ++j) {
            const double gj = gq[a * 3 + j];
            gu[0][j] = fma(ue[a * 3], gj, gu[0][j]);
            gu[1][j] = fma(ue[a * 3 + 1], gj, gu[1][j]);
            gu[2][j] = fma(ue[a * 3 + 2], gj, gu[2][j]);
          }
        const double* so = NS ? g.state_old + (e * NQ + q) * NS : nullptr;
        double* sn = (NS && g.state_new) ? g.state_new + (e * NQ + q) * NS : nullptr;
        double P9[9], scr[Model::SCR];
        Model::point(g.props, gu, s_jxw[q], so, sn, P9, scr);
#pragma unroll
        for (int m = 0; m < 9; ++m) P2[m] = df64_split(P9[m]);
        if (WANT_K) {
          Model::split_scratch(scr, scr2);
          bnd = Model::abound(scr2) * 1.0001f;
        }
      } else {
        for (int m = 0; m < 9; ++m) P2[m] = make_float2(0.f, 0.f);
        if (WANT_K)
          for (int m = 0; m < Model::SCR2; ++m) scr2[m] = make_float2(0.f, 0.f);
      }
      s_bnd[tid] = bnd;
    }
    __syncthreads();
    // the 45 unique JxW A entries of every point in double-float, on all threads:
    // entry w = (r1, r2), r1 = 3i + J <= r2 = 3k + L, in row order
    if (WANT_K) {
      for (int idx = tid; idx < NPT * 45; idx += NTHR) {
        const int pt = idx / 45, w = idx - pt * 45;
        int r1 = 0, m = w;
        while (m >= 9 - r1) {
          m -= 9 - r1;
          ++r1;
        }
        const int r2 = r1 + m;
        s_ent[idx] = Model::aentry_df64(s_scr2 + pt * SCR2_MAX, r1 / 3, r1 % 3, r2 / 3, r2 % 3);
      }
    }
    if (WANT_K && tid < EPT) {  // the element's scale 2^tau > |every tangent entry|
      float b = 0.f;
      for (int q = 0; q < NQ; ++q) b = fmaxf(b, s_bnd[tid * NQ + q]);
      int tau = 0;
      if (b > 0.f) frexpf(b, &tau);
      s_tau[tid] = tau < -119 ? -119 : (tau > 126 ? 126 : tau);
    }
    if (WANT_R) {  // R_(a,i) = sum_q sum_J dNX_qaJ P_q,iJ in double-float, q in order
      for (int i = tid; i < EPT * NDOF; i += NTHR) {
        const int el = i / NDOF, r = i - el * NDOF, a = r / 3, ii = r - a * 3;
        const int64_t e = tile_elem(c, u, el, P);
        if (e >= g.ne) continue;
        float2 R = make_float2(0.f, 0.f);
        for (int q = 0; q < NQ; ++q) {
          const float2* gq = s_g2 + (q * A + a) * 3;
          const float2* Pq = s_P2 + (el * NQ + q) * 9 + ii * 3;
          R = df64_dot3_acc(R, gq[0], Pq[0], gq[1], Pq[1], gq[2], Pq[2]);
        }
        static_cast<double*>(g.Re)[e * NDOF + r] = widen(R.x) + widen(R.y);
      }
    }
    __syncthreads();
    if (!WANT_K) continue;
    // ---- A digit slices of the three K steps: thread (row m, half h), 8 columns each ----
    {
      const int m = tid >> 1, h = tid & 1, rq = m & 31;
      if (rq < 27) {
        const int el = 3 * (m >> 5) + rq / 9, ik = rq % 9, i = ik / 3, k = ik % 3;
        const float fs = pow2f(7 - s_tau[el]);
        const float2* ent = s_ent + el * NQ * 45;
        for (int ks = 0; ks < KS; ++ks) {
          uint32_t dig[ND][4];
#pragma unroll
          for (int cp = 0; cp < 4; ++cp) {
            uint32_t lo16[ND], hi16[ND];
#pragma unroll
            for (int half2 = 0; half2 < 2; ++half2) {
              const int r = 16 * ks + 8 * h + 2 * cp + half2;
              float xh = 0.f, xl = 0.f;
              if (r < KR) {
                const int q = r / 9, JL = r - q * 9;
                const int ra = 3 * i + JL / 3, rb = 3 * k + JL % 3;  // A_iJkL = A_kLiJ
                const int r1 = ra < rb ? ra : rb, r2 = ra < rb ? rb : ra;
                const float2 x = ent[q * 45 + r1 * 9 - (r1 * (r1 - 1)) / 2 + (r2 - r1)];
                xh = x.x * fs;
                xl = x.y * fs;
              }
#pragma unroll
              for (int d = 0; d < ND; ++d) {
                const float dh = rintf(xh), dl = rintf(xl);
                xh = (xh - dh) * 256.f;
                xl = (xl - dl) * 256.f;
                const uint32_t bits = __float_as_uint(dh + dl) >> 16;
                if (half2 == 0) lo16[d] = bits;
                else hi16[d] = bits;
              }
            }
#pragma unroll
            for (int d = 0; d < ND; ++d) dig[d][cp] = lo16[d] | (hi16[d] << 16);
          }
#pragma unroll
          for (int d = 0; d < ND; ++d)
            *reinterpret_cast<uint4*>(sm + S_A + ks * A_STEP + d * A_SLICE + op16(m, 8 * h)) =
                make_uint4(dig[d][0], dig[d][1], dig[d][2], dig[d][3]);
        }
      }
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    if (tid == 0) {
      if (wpend) {
        if (!mbar_wait(wbar, wph, budget)) {  // report, then wait the copy out
          atomicExch(err, 1);
          mbar_wait(wbar, wph, WAIT_BUDGET);
        }
        wph ^= 1u;
        wpend = false;
      }
      tc_fence_after();
#pragma unroll 1
      for (int ks = 0; ks < KS; ++ks)
#pragma unroll 1
        for (int gi = 0; gi < NGROUP; ++gi) {
          const int tt = kGroups[gi][0], sg = kGroups[gi][1], ns = kGroups[gi][2];
          const uint64_t ad = smem_desc(s0 + uint32_t(S_A + ks * A_STEP + tt * A_SLICE), 128, 256);
          const uint64_t bd = smem_desc(s0 + uint32_t(S_W + ks * W_STEP + sg * W_SLICE), 128, 256);
          mma_bf16(tmem + uint32_t((sg + tt) * NPAD), ad, bd, idesc_bf16(128, NPAD * ns),
                   (tt == 0 && ks == 0) ? 0u : 1u);
        }
      mma_commit(mbar);
    }
    {
      const bool ok = mbar_wait(mbar, mph, budget);
      if (__syncthreads_or(!ok)) {
        failed = true;
        break;
      }
      mph ^= 1u;
    }
    tc_fence_after();
    // ---- epilogue: levels -> double-float pairs, the symmetric half of K_e ----
    {
      const int qd = warp & 3, ch = warp >> 2;
      const int j = lane / 9, ik = lane - 9 * j;
      const int el = 3 * qd + (lane < 27 ? j : 0);
      const int64_t e = tile_elem(c, u, el, P);
      const bool mine = lane < 27 && e < g.ne;
      const float f1 = pow2f(s_tau[el] - 7);
      float2* dst = static_cast<float2*>(g.Ke) + e * (NP * 9) + ik;
#pragma unroll 1
      for (int n0 = ch * (NPAD / 2); n0 < (ch + 1) * (NPAD / 2); n0 += 4) {
        float v[NLEV][4];
        tmem_ld4x7(tmem + (uint32_t(32 * qd) << 16) + uint32_t(n0), v);
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) {
          const int n = n0 + jj;
          // sum_L v_L 2^(-8L): levels 6..4 in FP32 (their rounding is below 2^-55 of
          // level 0), then 3..0 in double-float
          float hi = fmaf(fmaf(v[6][jj], 0.00390625f, v[5][jj]), 0.00390625f, v[4][jj]), lo = 0.f;
#pragma unroll
          for (int Lv = 3; Lv >= 0; --Lv) {
            const float a = v[Lv][jj], b = hi * 0.00390625f;
            lo *= 0.00390625f;
            const float s1 = a + b, bb = s1 - a;
            lo += (a - (s1 - bb)) + (b - bb);
            hi = s1 + lo;
            lo = lo - (hi - s1);
          }
          if (mine && n < NP) {
            const float f = f1 * pow2f(s_sig[n] - 7);
            dst[n * 9] = make_float2(hi * f, lo * f);
          }
        }
      }
    }
    tc_fence_before();
    __syncthreads();
  }
  if (failed) {
    // one more bounded wait on the pending phases (a phase that already completed
    // returns at once), so that no MMA or copy is left in flight
    if (tid == 0) {
      atomicExch(err, 1);
      if (wpend) mbar_wait(wbar, wph, WAIT_BUDGET);
    }
    mbar_wait(mbar, mph, WAIT_BUDGET);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, 512);
  }
}

template <class Model, bool R, bool K>
cudaError_t go(const ElemArgs& a, int* err, cudaStream_t s) {
  cudaError_t e = ensure_smem<class_tc64_kernel<Model, R, K>>(size_t(SMEM));
  if (e != cudaSuccess) return e;
  const int64_t tiles = (a.ne + EPT - 1) / EPT + 8;
  const int64_t cap = num_sms();
  const unsigned grid = unsigned(tiles < cap ? tiles : cap);
  class_tc64_kernel<Model, R, K><<<grid, NTHR, SMEM, s>>>(a, err);
  return cudaGetLastError();
}

template <class Model>
cudaError_t launch(bool want_r, bool want_k, const ElemArgs& a, int* err, cudaStream_t s, int* launches) {
  if (a.ne <= 0 || (!want_r && !want_k)) return cudaSuccess;
  ++*launches;
  if (!want_k) return go<Model, true, false>(a, err, s);
  return want_r ? go<Model, true, true>(a, err, s) : go<Model, false, true>(a, err, s);
}

// Host: the FP64 section of one class, from its spatial gradients and weights.
bool section(const std::vector<double>& dnx, const std::vector<double>& jxw, unsigned char* out) {
  int32_t sig[NPAD] = {0};
  for (int a = 0, n = 0; a < A; ++a)
    for (int b = a; b < A; ++b, ++n) {
      double w[KR], mx = 0.0;
      for (int r = 0; r < KR; ++r) {
        const int q = r / 9, J = (r % 9) / 3, Lc = r % 3;
        w[r] = dnx[(q * A + a) * 3 + J] * dnx[(q * A + b) * 3 + Lc];
        mx = std::fmax(mx, std::fabs(w[r]));
      }
      int ex = 0;
      if (mx > 0.0) std::frexp(mx, &ex);  // |w| < 2^ex
      if (ex < -119 || ex > 134) return false;  // the epilogue scales by 2^(ex - 7) in FP32
      sig[n] = ex;
      for (int r = 0; r < KR; ++r) {
        double y = std::ldexp(w[r], 7 - ex);  // |y| < 128, exact
        for (int d = 0; d < ND; ++d) {
          const double dd = std::nearbyint(y);
          y = (y - dd) * 256.0;
          const float fd = float(dd);
          uint32_t bits;
          std::memcpy(&bits, &fd, 4);
          const uint16_t b16 = uint16_t(bits >> 16);
          std::memcpy(out + C_W + (r / 16) * W_STEP + d * W_SLICE + op16(n, r % 16), &b16, 2);
        }
      }
    }
  std::memcpy(out + C_SIG, sig, sizeof sig);
  std::memcpy(out + C_G, dnx.data(), sizeof(double) * dnx.size());
  std::memcpy(out + C_JXW, jxw.data(), sizeof(double) * jxw.size());
  return true;
}
}  // namespace x64

// ---- host: the class table ---------------------------------------------------------
// tf32 with round-to-nearest, ties away (the device's cvt.rna.tf32.f32)
float tf32_rna_host(float x) {
  uint32_t b;
  std::memcpy(&b, &x, 4);
  if ((b & 0x7F800000u) != 0x7F800000u) b = (b + 0x1000u) & 0xFFFFE000u;
  float r;
  std::memcpy(&r, &b, 4);
  return r;
}

template <int ET>
bool table(int P, const double* xc, const double* ref, std::vector<unsigned char>& out) {
  using G = L<ET>;
  constexpr int A = G::A, NQ = G::NQ;
  const double* N = ref;
  const double* dN = ref + NQ * A;
  const double* w = dN + NQ * A * 3;
  (void)N;
  // header: class count, offset of the FP32-element section, of the FP64 section (tet10: the
  // exact-digit operands and gradients; hex27: the gradients the double-float kernel reads)
  constexpr size_t C64 = ET == 7 ? size_t(x64::C_BYTES) : size_t(HEX27_CLASS_BYTES);
  const int off32 = HEADER, off64 = HEADER + P * G::CLASS_BYTES;
  out.assign(size_t(off64) + size_t(P) * C64, 0);
  const int hdr[3] = {P, off32, off64};
  std::memcpy(out.data(), hdr, sizeof hdr);
  std::vector<double> dnx(size_t(NQ) * A * 3), jxw(NQ);
  for (int c = 0; c < P; ++c) {
    const double* X = xc + size_t(c) * A * 3;
    for (int q = 0; q < NQ; ++q) {
      double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
      for (int a = 0; a < A; ++a)
        for (int d = 0; d < 3; ++d)
          for (int k = 0; k < 3; ++k) J[d][k] += X[a * 3 + d] * dN[(q * A + a) * 3 + k];
      const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1], c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2],
                   c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
      const double det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
      if (!(det > 0.0) || !std::isfinite(det)) return false;
      double inv[3][3];
      inv[0][0] = c00 / det;
      inv[1][0] = c01 / det;
      inv[2][0] = c02 / det;
      inv[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;
      inv[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
      inv[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;
      inv[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
      inv[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;
      inv[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
      // dNX_a = dN_xi_a J^-1 (J[d][k] = dX_d / dxi_k)
      for (int a = 0; a < A; ++a)
        for (int j = 0; j < 3; ++j) {
          double s = 0.0;
          for (int k = 0; k < 3; ++k) s += dN[(q * A + a) * 3 + k] * inv[k][j];
          dnx[(q * A + a) * 3 + j] = s;
        }
      jxw[q] = det * w[q];
    }
    unsigned char* cb = out.data() + HEADER + size_t(c) * G::CLASS_BYTES;
    for (int s = 0; s < G::KSTEPS; ++s) {
      unsigned char* hi = cb + size_t(s) * G::W_STEP;
      unsigned char* lo = hi + G::W_TERM;
      for (int n = 0; n < G::NP; ++n) {
        int a = 0, m = n;
        while (m >= A - a) {
          m -= A - a;
          ++a;
        }
        const int b = a + m;
        for (int kk = 0; kk < 8; ++kk) {
          const int r = 8 * s + kk;
          if (r >= G::KR) continue;
          const int q = r / 9, J = (r % 9) / 3, Lc = r % 3;
          const float v = float(dnx[(q * A + a) * 3 + J] * dnx[(q * A + b) * 3 + Lc]);
          const float h = tf32_rna_host(v), l = v - h;
          const size_t off = size_t(n >> 3) * 256 + size_t(kk >> 2) * 128 + size_t(n & 7) * 16 + size_t(kk & 3) * 4;
          std::memcpy(hi + off, &h, 4);
          std::memcpy(lo + off, &l, 4);
        }
      }
    }
    float* gb = reinterpret_cast<float*>(cb + size_t(G::KSTEPS) * G::W_STEP);
    for (int i = 0; i < NQ * A * 3; ++i) gb[i] = float(dnx[i]);
    for (int q = 0; q < NQ; ++q) gb[NQ * A * 3 + q] = float(jxw[q]);
    if (ET == 7 && !x64::section(dnx, jxw, out.data() + off64 + size_t(c) * C64)) return false;
    if (ET == 8) {
      std::memcpy(out.data() + off64 + size_t(c) * C64, dnx.data(), sizeof(double) * dnx.size());
      std::memcpy(out.data() + off64 + size_t(c) * C64 + sizeof(double) * dnx.size(), jxw.data(),
                  sizeof(double) * jxw.size());
    }
  }
  return true;
}

}  // namespace ctc

bool class_tc_table(int elem_type, int nclass, const double* xc, const double* ref, std::vector<unsigned char>& out) {
  if (nclass < 1 || nclass > 8) return false;
  if (elem_type == 7) return ctc::table<7>(nclass, xc, ref, out);
  if (elem_type == 8) return ctc::table<8>(nclass, xc, ref, out);
  return false;
}

bool class_tc_enabled() {
  const char* v = std::getenv("FEC_CLASS_TC");
  return !(v && v[0] == '0');
}

bool class_tc_runs(int physics, int elem_type, int precision, bool want_r, bool want_k, bool has_table) {
  if (!has_table || !(want_r || want_k) || (physics != 2 && physics != 3) || !class_tc_enabled()) return false;
  if (precision == 1) return elem_type == 7 || (elem_type == 8 && !hex27_on_cuda_cores());
  return precision == 0 && elem_type == 7;  // FP64: tet10 (the exact digit levels hold 36 reduction terms)
}

cudaError_t launch_class_tc(int physics, int elem_type, int precision, bool want_r, bool want_k, const ElemArgs& a,
                            cudaStream_t s, int* launches) {
  int* err = a.wait_err;
  if (!err) {
    const cudaError_t e = wait_error_flag(&err);
    if (e != cudaSuccess) return e;
  }
  if (precision == 0) {
    if (elem_type != 7) return cudaErrorNotSupported;
    if (physics == 2) return ctc::x64::launch<NeoHookean>(want_r, want_k, a, err, s, launches);
    if (physics == 3) return ctc::x64::launch<J2>(want_r, want_k, a, err, s, launches);
    return cudaErrorNotSupported;
  }
  if (elem_type == 7) {
    if (physics == 2) return ctc::launch<7, NeoHookean>(want_r, want_k, a, err, s, launches);
    if (physics == 3) return ctc::launch<7, J2>(want_r, want_k, a, err, s, launches);
  } else if (elem_type == 8) {
    if (physics == 2) return ctc::launch<8, NeoHookean>(want_r, want_k, a, err, s, launches);
    if (physics == 3) return ctc::launch<8, J2>(want_r, want_k, a, err, s, launches);
  }
  return cudaErrorNotSupported;
}

}  // namespace fec
