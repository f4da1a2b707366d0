// fec_gather.cu -- instantiations of the node gather and the mechanics
// dispatcher, plus the reference-element tables.
#include <cmath>
#include <cstdlib>
#include "fec_launch.h"

namespace fec {

cudaError_t launch_mech_neohookean(int, int, bool, bool, const ElemArgs&, cudaStream_t, int*);
cudaError_t launch_mech_j2(int, int, bool, bool, const ElemArgs&, cudaStream_t, int*);
cudaError_t launch_mech_j2mlp(int, int, bool, bool, const ElemArgs&, cudaStream_t, int*);

cudaError_t launch_mech(int physics, int elem_type, int precision, bool want_r, bool want_k, const ElemArgs& a,
                        cudaStream_t s, int* launches) {
  if (physics == 2) return launch_mech_neohookean(elem_type, precision, want_r, want_k, a, s, launches);
  if (physics == 3) return launch_mech_j2(elem_type, precision, want_r, want_k, a, s, launches);
  if (physics == 4) return launch_mech_j2mlp(elem_type, precision, want_r, want_k, a, s, launches);
  return cudaErrorNotSupported;
}

namespace {
constexpr int WPB = 8;

// Gather variants: (min blocks per SM, values in flight per lane).  Variant 0
// favours occupancy, variant 1 favours loads in flight per warp.
int gather_variant() {
  static int v = [] {
    const char* e = getenv("FEC_GATHER_VARIANT");
    return e ? atoi(e) : 0;
  }();
  return v;
}

template <typename Real, int NF, int A, int MINB, int BUDGET>
cudaError_t go1(const GatherArgs& g, cudaStream_t s, int* launches) {
  const size_t smem = sizeof(float) * GatherAcc::WORDS * size_t(WPB) * size_t(g.acc_stride);
  auto kern = node_gather_kernel<Real, NF, A, WPB, MINB, BUDGET>;
  cudaError_t err = ensure_smem<node_gather_kernel<Real, NF, A, WPB, MINB, BUDGET>>(smem);
  if (err != cudaSuccess) return err;
  const int64_t count = g.nodes ? g.nnodes : g.nn;
  const unsigned grid = unsigned((count + WPB - 1) / WPB);
  kern<<<grid, WPB * 32, smem, s>>>(g);
  ++*launches;
  return cudaGetLastError();
}

// Hex27 nodes gather 243 values per element: with the default budget a warp has
// one element's loads in flight.  For the double-float (FP64) workspace, two CTAs
// per SM (128 registers) and a budget of two elements' loads instead (batched
// mixed mesh: the FP64 gathers 10.8 -> 10.2 ms; the same for the FP32 workspace
// was slower, 9.4 -> 9.7 ms); FEC_GATHER_HEX27=narrow keeps the default (bitwise
// the same results).
bool gather_hex27_wide() {
  const char* e = getenv("FEC_GATHER_HEX27");
  return !(e && e[0] == 'n');
}

template <typename Real, int NF, int A>
cudaError_t go(const GatherArgs& g, cudaStream_t s, int* launches) {
  if ((g.nodes ? g.nnodes : g.nn) <= 0) return cudaSuccess;
  if constexpr (A == 27 && sizeof(Real) == 8) {
    if (gather_hex27_wide()) return go1<Real, NF, 27, 2, 16>(g, s, launches);
  }
  if (gather_variant() == 1) return go1<Real, NF, A, 2, sizeof(Real) == 8 ? 12 : 18>(g, s, launches);
  return go1<Real, NF, A, 3, sizeof(Real) == 8 ? 6 : 12>(g, s, launches);
}

// The software-pipelined hex8 gather: one block of hex8 mechanics elements in
// the node-rows layout (or the FP64 pair layout), stiffness wanted.  FEC_GATHER_PIPE=0 keeps the
// one-warp-per-node kernel (bitwise the same results).
bool gather_pipe_enabled() {
  const char* e = getenv("FEC_GATHER_PIPE");
  return !(e && e[0] == '0');
}

template <typename Real, bool PAIRS = false>
cudaError_t go_pipe(const GatherArgs& g, cudaStream_t s, int* launches) {
  constexpr int MINB = 2;
  const size_t acc_bytes = (size_t(g.acc_stride) * GatherAcc::WORDS * sizeof(float) + 15) / 16 * 16;
  const size_t smem = size_t(gp::WPB) * (acc_bytes + 2 * gp::Stage<Real, PAIRS>::BYTES);
  cudaError_t err = ensure_smem<node_gather_hex8_pipe_kernel<Real, MINB, PAIRS>>(smem);
  if (err != cudaSuccess) return err;
  const int64_t need = (g.nn + gp::WPB - 1) / gp::WPB;
  const int64_t cap = int64_t(num_sms()) * MINB;
  const unsigned grid = unsigned(need < cap ? need : cap);
  node_gather_hex8_pipe_kernel<Real, MINB, PAIRS><<<grid, gp::WPB * 32, smem, s>>>(g);
  ++*launches;
  return cudaGetLastError();
}

template <typename Real, int NF>
cudaError_t by_size(const GatherArgs& g, cudaStream_t s, int* launches) {
  if (NF == 3 && g.nn > 0 && g.nblocks == 1 && g.blk[0].nnpe == 8 && g.nzval != nullptr && gather_pipe_enabled()) {
    if (g.blk[0].layout == KE_NODE_ROWS) return go_pipe<Real>(g, s, launches);
    if constexpr (sizeof(Real) == 8)
      if (g.blk[0].layout == KE_PAIRS) return go_pipe<Real, true>(g, s, launches);
  }
  int A = g.blk[0].nnpe;
  for (int b = 1; b < g.nblocks; ++b)
    if (g.blk[b].nnpe != A) A = 0;
  switch (A) {
    case 8: return go<Real, NF, 8>(g, s, launches);
    case 4: return go<Real, NF, 4>(g, s, launches);
    case 10: return go<Real, NF, 10>(g, s, launches);
    case 27: return go<Real, NF, 27>(g, s, launches);
    default: return go<Real, NF, 0>(g, s, launches);
  }
}
template <typename Real, int NF>
cudaError_t groups(const GatherArgs& g0, const int32_t* nodes, const NodeGroup* grp, int ngroups, cudaStream_t s,
                   int* launches) {
  for (int i = 0; i < ngroups; ++i) {
    GatherArgs g = g0;
    g.nodes = nodes + grp[i].off;
    g.nnodes = grp[i].count;
    cudaError_t e;
    switch (grp[i].A) {
      case 4: e = go<Real, NF, 4>(g, s, launches); break;
      case 8: e = go<Real, NF, 8>(g, s, launches); break;
      case 10: e = go<Real, NF, 10>(g, s, launches); break;
      case 27: e = go<Real, NF, 27>(g, s, launches); break;
      default: e = go<Real, NF, 0>(g, s, launches); break;
    }
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}
}  // namespace

cudaError_t launch_gather_groups(int precision, int nf, const GatherArgs& g, const int32_t* nodes,
                                 const NodeGroup* grp, int ngroups, cudaStream_t s, int* launches) {
  if (precision == 0) {
    if (nf == 1) return groups<float2, 1>(g, nodes, grp, ngroups, s, launches);
    if (nf == 3) return groups<float2, 3>(g, nodes, grp, ngroups, s, launches);
  } else if (precision == 1) {
    if (nf == 1) return groups<float, 1>(g, nodes, grp, ngroups, s, launches);
    if (nf == 3) return groups<float, 3>(g, nodes, grp, ngroups, s, launches);
  }
  return cudaErrorNotSupported;
}

cudaError_t launch_gather(int precision, int nf, const GatherArgs& g, cudaStream_t s, int* launches) {
  if (precision == 0) {  // FP64 kernels leave double-float workspace entries
    if (nf == 1) return by_size<float2, 1>(g, s, launches);
    if (nf == 3) return by_size<float2, 3>(g, s, launches);
  } else if (precision == 1) {
    if (nf == 1) return by_size<float, 1>(g, s, launches);
    if (nf == 3) return by_size<float, 3>(g, s, launches);
  }
  return cudaErrorNotSupported;
}

int elem_nnpe(int et) {
  switch (et) { case 1: return 8; case 2: return 4; case 6: return 4; case 7: return 10; case 8: return 27; }
  return 0;
}
int num_sms() {
  static int count[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 148;
  if (!count[dev]) cudaDeviceGetAttribute(&count[dev], cudaDevAttrMultiProcessorCount, dev);
  return count[dev] > 0 ? count[dev] : 148;
}

bool hex8_df64_tile_kernel() {
  const char* v = std::getenv("FEC_HEX8_DF64");
  return v && v[0] == 't';
}

int elem_dim(int et) {
  switch (et) { case 1: case 6: case 7: case 8: return 3; case 2: return 2; }
  return 0;
}
int elem_nq(int et) {
  switch (et) { case 1: return 8; case 2: return 4; case 6: return 1; case 7: return 4; case 8: return 27; }
  return 0;
}

// Lagrange shape functions and quadrature rules of the reference elements on
// the path (the rules ReferenceFiniteElements.jl supplies to
// src/FunctionSpaces.jl:104-126): Q1 quad/hex with the 2-point Gauss-Legendre
// tensor rule, P1 tet with its 1-point rule, P2 tet (exodus TETRA10 node order)
// with the 4-point rule, Q2 hex with the 3-point Gauss-Legendre tensor rule.
int ref_tables(int et, double* out, int cap) {
  const int A = elem_nnpe(et), D = elem_dim(et), NQ = elem_nq(et);
  if (!A) return 0;
  const int size = NQ * A + NQ * A * D + NQ;
  if (size > cap) return 0;
  double* N = out;
  double* dN = out + NQ * A;
  double* w = dN + NQ * A * D;
  const double g = 1.0 / std::sqrt(3.0);
  if (et == 2) {
    const double xi[4][2] = {{-1, -1}, {1, -1}, {1, 1}, {-1, 1}};
    for (int q = 0; q < 4; ++q) {
      const double s = (q & 1) ? g : -g, t = (q & 2) ? g : -g;
      w[q] = 1.0;
      for (int a = 0; a < 4; ++a) {
        N[q * 4 + a] = 0.25 * (1 + xi[a][0] * s) * (1 + xi[a][1] * t);
        dN[(q * 4 + a) * 2 + 0] = 0.25 * xi[a][0] * (1 + xi[a][1] * t);
        dN[(q * 4 + a) * 2 + 1] = 0.25 * xi[a][1] * (1 + xi[a][0] * s);
      }
    }
  } else if (et == 1) {
    const double xi[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                             {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
    for (int q = 0; q < 8; ++q) {
      const double s = (q & 1) ? g : -g, t = (q & 2) ? g : -g, u = (q & 4) ? g : -g;
      w[q] = 1.0;
      for (int a = 0; a < 8; ++a) {
        const double fs = 1 + xi[a][0] * s, ft = 1 + xi[a][1] * t, fu = 1 + xi[a][2] * u;
        N[q * 8 + a] = 0.125 * fs * ft * fu;
        dN[(q * 8 + a) * 3 + 0] = 0.125 * xi[a][0] * ft * fu;
        dN[(q * 8 + a) * 3 + 1] = 0.125 * xi[a][1] * fs * fu;
        dN[(q * 8 + a) * 3 + 2] = 0.125 * xi[a][2] * fs * ft;
      }
    }
  } else if (et == 6) {
    w[0] = 1.0 / 6.0;
    const double dl[4][3] = {{-1, -1, -1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    for (int a = 0; a < 4; ++a) {
      N[a] = 0.25;
      for (int k = 0; k < 3; ++k) dN[a * 3 + k] = dl[a][k];
    }
  } else if (et == 7) {
    const double al = (5.0 + 3.0 * std::sqrt(5.0)) / 20.0, be = (5.0 - std::sqrt(5.0)) / 20.0;
    const double pts[4][3] = {{be, be, be}, {al, be, be}, {be, al, be}, {be, be, al}};
    const double dl[4][3] = {{-1, -1, -1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    const int ed[6][2] = {{0, 1}, {1, 2}, {0, 2}, {0, 3}, {1, 3}, {2, 3}};
    for (int q = 0; q < 4; ++q) {
      w[q] = 1.0 / 24.0;
      const double l[4] = {1 - pts[q][0] - pts[q][1] - pts[q][2], pts[q][0], pts[q][1], pts[q][2]};
      for (int v = 0; v < 4; ++v) {
        N[q * 10 + v] = l[v] * (2 * l[v] - 1);
        for (int k = 0; k < 3; ++k) dN[(q * 10 + v) * 3 + k] = (4 * l[v] - 1) * dl[v][k];
      }
      for (int e = 0; e < 6; ++e) {
        const int i = ed[e][0], j = ed[e][1];
        N[q * 10 + 4 + e] = 4 * l[i] * l[j];
        for (int k = 0; k < 3; ++k) dN[(q * 10 + 4 + e) * 3 + k] = 4 * (dl[i][k] * l[j] + l[i] * dl[j][k]);
      }
    }
  } else if (et == 8) {
    const double p = std::sqrt(0.6);
    const double gp[3] = {-p, 0.0, p}, gw[3] = {5.0 / 9.0, 8.0 / 9.0, 5.0 / 9.0};
    auto lag = [](double x, double* v, double* d) {
      v[0] = 0.5 * x * (x - 1.0); d[0] = x - 0.5;
      v[1] = 1.0 - x * x;         d[1] = -2.0 * x;
      v[2] = 0.5 * x * (x + 1.0); d[2] = x + 0.5;
    };
    for (int q = 0; q < 27; ++q) {
      const int qx = q % 3, qy = (q / 3) % 3, qz = q / 9;
      w[q] = gw[qx] * gw[qy] * gw[qz];
      double vx[3], dx[3], vy[3], dy[3], vz[3], dz[3];
      lag(gp[qx], vx, dx); lag(gp[qy], vy, dy); lag(gp[qz], vz, dz);
      for (int a = 0; a < 27; ++a) {
        const int i = a % 3, j = (a / 3) % 3, k = a / 9;
        N[q * 27 + a] = vx[i] * vy[j] * vz[k];
        dN[(q * 27 + a) * 3 + 0] = dx[i] * vy[j] * vz[k];
        dN[(q * 27 + a) * 3 + 1] = vx[i] * dy[j] * vz[k];
        dN[(q * 27 + a) * 3 + 2] = vx[i] * vy[j] * dz[k];
      }
    }
  }
  return size;
}

}  // namespace fec
