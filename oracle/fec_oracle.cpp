// fec_oracle.cpp -- TEST INFRASTRUCTURE ONLY.
//
// CPU restatement of FiniteElementContainers.jl's assembly path, used by the
// tests, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg as the
// checker.  Nothing in the product links or calls this file.
//
// What it restates (reference paths are relative to the FiniteElementContainers.jl
// project root):
//   * structured hex8 / quad4 meshes ......... src/meshes/StructuredMesh.jl:85-131, 233-250, 433-470
//   * nodesets of a structured hex8 mesh ..... src/meshes/StructuredMesh.jl:452-470
//   * DofManager numbering ................... src/DofManagers.jl:227-298
//   * element-ordered COO pattern ............ src/assemblers/SparsityPatterns.jl:160-231
//   * the per-element quadrature loop ........ src/assemblers/Assemblers.jl:402-432
//   * residual scatter ....................... src/assemblers/Assemblers.jl:72-87, src/Utils.jl:1-21
//   * element matrix -> COO slot storage ..... src/assemblers/Assemblers.jl:109-124
//   * COO -> CSC with duplicate summation .... SparseArrays.sparse! as called at
//                                              src/assemblers/SparsityPatterns.jl:301-308
//   * Poisson physics ........................ test/poisson/TestPoissonCommon.jl:75-107
//   * mechanics residual/tangent shape ....... test/mechanics/TestMechanicsCommon.jl:140-190,
//                                              src/Formulations.jl:462-576
//   * compressible Neo-Hookean energy ........ test/mechanics/TestMechanicsLargeDeformation.jl:17-27
//   * J2 plasticity (absent from the reference; classical radial return with
//     linear isotropic hardening, Simo & Hughes 1998 Box 3.2)
//
// Third-party arithmetic restated here: ReferenceFiniteElements.jl (Lagrange
// shape functions, tensor-product Gauss-Legendre 2-point rule, isoparametric map)
// and Tensors.jl (the gradient/hessian of the energy, written out analytically).
//
// Parity pins: the Poisson quad4 path reproduces test/poisson/poisson.gold; the
// mesh/connectivity restatement reproduces test/TestMesh.jl and test/TestFields.jl
// known answers.  Neo-Hookean and J2: parity unpinned (no reference test runs them).
//
// All index arguments follow the reference: 1-based Int64.

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef int64_t i64;

extern "C" {

// ---------------------------------------------------------------------------
// Meshes (StructuredMesh.jl)
// ---------------------------------------------------------------------------

// LinRange(a, b, n)[k], k 1-based, evaluated as Julia's LinRange does:
// t = (k-1)/(n-1); (1-t)*a + t*b
static double linrange(double a, double b, i64 n, i64 k) {
  if (n == 1) return a;
  const double t = double(k - 1) / double(n - 1);
  return (1.0 - t) * a + t * b;
}

// counts = nodes per direction.  coords: 3 x NN column-major; conns: 8 x NE column-major.
// StructuredMesh.jl:85-131 (element loop ex outer, ey, ez inner) and :433-449.
void orc_structured_hex8(i64 Nx, i64 Ny, i64 Nz, const double* mins, const double* maxs,
                         double* coords, i64* conns) {
  // _three_dimensional_coords!: outer loop bound counts[1] for z and counts[3] for x
  const i64 c1 = Nx, c2 = Ny, c3 = Nz;
  i64 n = 0;
  for (i64 nz = 1; nz <= c1; ++nz)
    for (i64 ny = 1; ny <= c2; ++ny)
      for (i64 nx = 1; nx <= c3; ++nx) {
        coords[3 * n + 0] = linrange(mins[0], maxs[0], c1, nx);
        coords[3 * n + 1] = linrange(mins[1], maxs[1], c2, ny);
        coords[3 * n + 2] = linrange(mins[2], maxs[2], c3, nz);
        ++n;
      }
  auto node = [&](i64 i, i64 j, i64 k) { return i + Nx * (j - 1) + Nx * Ny * (k - 1); };
  i64 e = 0;
  for (i64 ex = 1; ex <= Nx - 1; ++ex)
    for (i64 ey = 1; ey <= Ny - 1; ++ey)
      for (i64 ez = 1; ez <= Nz - 1; ++ez) {
        i64* c = conns + 8 * e;
        c[0] = node(ex, ey, ez);
        c[1] = node(ex + 1, ey, ez);
        c[2] = node(ex + 1, ey + 1, ez);
        c[3] = node(ex, ey + 1, ez);
        c[4] = node(ex, ey, ez + 1);
        c[5] = node(ex + 1, ey, ez + 1);
        c[6] = node(ex + 1, ey + 1, ez + 1);
        c[7] = node(ex, ey + 1, ez + 1);
        ++e;
      }
}

// StructuredMesh.jl:233-250 and the 2D coordinate loop.
void orc_structured_quad4(i64 Nx, i64 Ny, const double* mins, const double* maxs,
                          double* coords, i64* conns) {
  i64 n = 0;
  for (i64 ny = 1; ny <= Nx; ++ny)
    for (i64 nx = 1; nx <= Ny; ++nx) {
      coords[2 * n + 0] = linrange(mins[0], maxs[0], Nx, nx);
      coords[2 * n + 1] = linrange(mins[1], maxs[1], Ny, ny);
      ++n;
    }
  auto node = [&](i64 i, i64 j) { return i + (j - 1) * Nx; };
  i64 e = 0;
  for (i64 ex = 1; ex <= Nx - 1; ++ex)
    for (i64 ey = 1; ey <= Ny - 1; ++ey) {
      i64* c = conns + 4 * e;
      c[0] = node(ex, ey);
      c[1] = node(ex + 1, ey);
      c[2] = node(ex + 1, ey + 1);
      c[3] = node(ex, ey + 1);
      ++e;
    }
}

// _three_dimensional_nsets (StructuredMesh.jl:452-470).  face: 0 bottom, 1 right,
// 2 front, 3 top, 4 left, 5 back.  Returns the count; writes 1-based node ids
// in the reference's comprehension order (first index fastest).
i64 orc_hex8_nodeset(i64 Nx, i64 Ny, i64 Nz, int face, i64* out) {
  auto node = [&](i64 i, i64 j, i64 k) { return i + (j - 1) * Nx + (k - 1) * Nx * Ny; };
  i64 n = 0;
  switch (face) {
    case 0: for (i64 k = 1; k <= Nz; ++k) for (i64 i = 1; i <= Nx; ++i) out[n++] = node(i, 1, k); break;
    case 1: for (i64 k = 1; k <= Nz; ++k) for (i64 j = 1; j <= Ny; ++j) out[n++] = node(Nx, j, k); break;
    case 2: for (i64 j = 1; j <= Ny; ++j) for (i64 i = 1; i <= Nx; ++i) out[n++] = node(i, j, Nz); break;
    case 3: for (i64 k = 1; k <= Nz; ++k) for (i64 i = 1; i <= Nx; ++i) out[n++] = node(i, Ny, k); break;
    case 4: for (i64 k = 1; k <= Nz; ++k) for (i64 j = 1; j <= Ny; ++j) out[n++] = node(1, j, k); break;
    case 5: for (i64 j = 1; j <= Ny; ++j) for (i64 i = 1; i <= Nx; ++i) out[n++] = node(i, j, 1); break;
    default: return -1;
  }
  return n;
}

// ---------------------------------------------------------------------------
// DofManager (DofManagers.jl:227-298, no periodic pairs)
// ---------------------------------------------------------------------------

// dirichlet: any order, duplicates allowed (dirichlet_dofs = unique(sort(...)),
// DirichletBCs.jl:396-398).  Writes unknown_dofs (sorted complement) and
// dof_to_unknown (rank, or -1 for a Dirichlet dof).  Returns n_unknowns, or -1
// when a dof is out of range (the reference asserts).
i64 orc_update_dofs(i64 ndofs, const i64* dirichlet, i64 nd, i64* unknown_dofs, i64* dof_to_unknown) {
  std::vector<char> fixed(ndofs, 0);
  for (i64 i = 0; i < nd; ++i) {
    if (dirichlet[i] < 1 || dirichlet[i] > ndofs) return -1;
    fixed[dirichlet[i] - 1] = 1;
  }
  i64 k = 0;
  for (i64 d = 1; d <= ndofs; ++d) {
    if (fixed[d - 1]) {
      dof_to_unknown[d - 1] = -1;
    } else {
      unknown_dofs[k] = d;
      dof_to_unknown[d - 1] = ++k;
    }
  }
  return k;
}

// ---------------------------------------------------------------------------
// Sparsity pattern (SparsityPatterns.jl:160-231)
// ---------------------------------------------------------------------------

// Counts the kept COO entries.  Blocks are given as nnpe[b], ne[b]; conn is
// the flat concatenation (Fields.jl:129-160).
i64 orc_pattern_count(int nblocks, const i64* nnpe, const i64* ne, const i64* conn, int ND,
                      const i64* dof_to_unknown) {
  i64 n = 0, off = 0;
  for (int b = 0; b < nblocks; ++b) {
    const i64 ndpe = ND * nnpe[b];
    std::vector<i64> dc(ndpe);
    for (i64 e = 0; e < ne[b]; ++e) {
      const i64* c = conn + off + e * nnpe[b];
      for (i64 a = 0; a < nnpe[b]; ++a)
        for (int d = 0; d < ND; ++d) dc[a * ND + d] = ND * (c[a] - 1) + d + 1;
      for (i64 i = 0; i < ndpe; ++i) {
        if (dof_to_unknown[dc[i] - 1] <= 0) continue;
        for (i64 j = 0; j < ndpe; ++j)
          if (dof_to_unknown[dc[j] - 1] > 0) ++n;
      }
    }
    off += nnpe[b] * ne[b];
  }
  return n;
}

// Is/Js = unknown indices; slots = 1-based raw slot into the element-ordered
// storage ((e-1)*NDOF^2 + (i-1)*NDOF + j, block-offset).
void orc_pattern_fill(int nblocks, const i64* nnpe, const i64* ne, const i64* conn, int ND,
                      const i64* dof_to_unknown, i64* Is, i64* Js, i64* slots) {
  i64 n = 0, off = 0, dof_num = 1;
  for (int b = 0; b < nblocks; ++b) {
    const i64 ndpe = ND * nnpe[b];
    std::vector<i64> dc(ndpe);
    for (i64 e = 0; e < ne[b]; ++e) {
      const i64* c = conn + off + e * nnpe[b];
      for (i64 a = 0; a < nnpe[b]; ++a)
        for (int d = 0; d < ND; ++d) dc[a * ND + d] = ND * (c[a] - 1) + d + 1;
      for (i64 i = 0; i < ndpe; ++i) {
        const i64 ri = dof_to_unknown[dc[i] - 1];
        for (i64 j = 0; j < ndpe; ++j) {
          const i64 rj = dof_to_unknown[dc[j] - 1];
          if (ri > 0 && rj > 0) {
            Is[n] = ri;
            Js[n] = rj;
            slots[n] = dof_num;
            ++n;
          }
          ++dof_num;
        }
      }
    }
    off += nnpe[b] * ne[b];
  }
}

// ---------------------------------------------------------------------------
// SparseArrays.sparse!(I, J, V, m, n, +): COO -> CSR (counting sort by row,
// entries kept in input order within a row), duplicates combined with + in
// input order (first value stored, later ones added), then CSR -> CSC by a
// counting sort on columns, which leaves rows ascending within each column.
// colptr (n+1), rowval, nzval are 1-based outputs; rowval/nzval must hold
// coo_len entries.  Returns nnz.
// ---------------------------------------------------------------------------
i64 orc_sparse_csc(i64 m, i64 n, i64 coo_len, const i64* I, const i64* J, const double* V,
                   i64* colptr, i64* rowval, double* nzval) {
  std::vector<i64> rowptr(m + 2, 0);
  for (i64 k = 0; k < coo_len; ++k) rowptr[I[k] + 1]++;
  rowptr[1] = 1;
  for (i64 i = 1; i <= m; ++i) rowptr[i + 1] += rowptr[i];  // rowptr[i] = start of row i (1-based)
  std::vector<i64> fill(rowptr.begin(), rowptr.end());
  std::vector<i64> csrcol(coo_len);
  std::vector<double> csrval(coo_len);
  for (i64 k = 0; k < coo_len; ++k) {
    const i64 p = fill[I[k]]++;
    csrcol[p - 1] = J[k];
    csrval[p - 1] = V[k];
  }
  // combine duplicates within each row, compacting in place
  std::vector<i64> lasttouch(n + 1, 0);
  std::vector<i64> crowptr(m + 2, 0);
  i64 w = 1;
  for (i64 i = 1; i <= m; ++i) {
    const i64 rs = rowptr[i], re = rowptr[i + 1];
    const i64 wstart = w;
    crowptr[i] = wstart;
    for (i64 p = rs; p < re; ++p) {
      const i64 j = csrcol[p - 1];
      const i64 lt = lasttouch[j];
      if (lt >= wstart) {
        csrval[lt - 1] = csrval[lt - 1] + csrval[p - 1];
      } else {
        csrcol[w - 1] = j;
        csrval[w - 1] = csrval[p - 1];
        lasttouch[j] = w;
        ++w;
      }
    }
  }
  crowptr[m + 1] = w;
  const i64 nnz = w - 1;
  // CSR -> CSC
  std::vector<i64> cnt(n + 2, 0);
  for (i64 p = 1; p <= nnz; ++p) cnt[csrcol[p - 1] + 1]++;
  colptr[0] = 1;
  for (i64 j = 1; j <= n; ++j) colptr[j] = colptr[j - 1] + cnt[j + 1];
  std::vector<i64> cfill(colptr, colptr + n + 1);
  for (i64 i = 1; i <= m; ++i)
    for (i64 p = crowptr[i]; p < crowptr[i + 1]; ++p) {
      const i64 j = csrcol[p - 1];
      const i64 q = cfill[j - 1]++;
      rowval[q - 1] = i;
      nzval[q - 1] = csrval[p - 1];
    }
  return nnz;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Reference elements (restating ReferenceFiniteElements.jl for the element
// types on the path) and the isoparametric map (MappedH1OrL2Interpolants).
// ---------------------------------------------------------------------------
namespace {

enum { ET_HEX8 = 1, ET_QUAD4 = 2, ET_TET4 = 6, ET_TET10 = 7, ET_HEX27 = 8 };

struct RefFE {
  int dim = 0, nnpe = 0, nq = 0;
  std::vector<double> N;    // [q][a]
  std::vector<double> dN;   // [q][a][k]
  std::vector<double> w;    // [q]
};

// 1D quadratic Lagrange on nodes -1, 0, 1 (in that order)
inline void lag2(double x, double* v, double* d) {
  v[0] = 0.5 * x * (x - 1.0); d[0] = x - 0.5;
  v[1] = 1.0 - x * x;         d[1] = -2.0 * x;
  v[2] = 0.5 * x * (x + 1.0); d[2] = x + 0.5;
}

RefFE make_ref(int et) {
  RefFE r;
  const double g = 1.0 / std::sqrt(3.0);
  if (et == ET_QUAD4) {
    r.dim = 2; r.nnpe = 4; r.nq = 4;
    const double xi[4][2] = {{-1, -1}, {1, -1}, {1, 1}, {-1, 1}};
    const double qp[4][2] = {{-g, -g}, {g, -g}, {-g, g}, {g, g}};
    for (int q = 0; q < 4; ++q) {
      r.w.push_back(1.0);
      for (int a = 0; a < 4; ++a) {
        const double s = qp[q][0], t = qp[q][1];
        r.N.push_back(0.25 * (1 + xi[a][0] * s) * (1 + xi[a][1] * t));
        r.dN.push_back(0.25 * xi[a][0] * (1 + xi[a][1] * t));
        r.dN.push_back(0.25 * xi[a][1] * (1 + xi[a][0] * s));
      }
    }
  } else if (et == ET_HEX8) {
    r.dim = 3; r.nnpe = 8; r.nq = 8;
    const double xi[8][3] = {{-1, -1, -1}, {1, -1, -1}, {1, 1, -1}, {-1, 1, -1},
                             {-1, -1, 1},  {1, -1, 1},  {1, 1, 1},  {-1, 1, 1}};
    for (int qz = 0; qz < 2; ++qz)
      for (int qy = 0; qy < 2; ++qy)
        for (int qx = 0; qx < 2; ++qx) {
          const double s = qx ? g : -g, t = qy ? g : -g, u = qz ? g : -g;
          r.w.push_back(1.0);
          for (int a = 0; a < 8; ++a) {
            const double fs = 1 + xi[a][0] * s, ft = 1 + xi[a][1] * t, fu = 1 + xi[a][2] * u;
            r.N.push_back(0.125 * fs * ft * fu);
            r.dN.push_back(0.125 * xi[a][0] * ft * fu);
            r.dN.push_back(0.125 * xi[a][1] * fs * fu);
            r.dN.push_back(0.125 * xi[a][2] * fs * ft);
          }
        }
  } else if (et == ET_TET4) {
    // one-point rule at the centroid, weight 1/6
    r.dim = 3; r.nnpe = 4; r.nq = 1;
    r.w.push_back(1.0 / 6.0);
    const double L = 0.25;
    r.N = {L, L, L, L};
    r.dN = {-1, -1, -1, 1, 0, 0, 0, 1, 0, 0, 0, 1};
  } else if (et == ET_TET10) {
    // four-point rule (a = (5+3 sqrt5)/20, b = (5-sqrt5)/20), weight 1/24 each
    r.dim = 3; r.nnpe = 10; r.nq = 4;
    const double a = (5.0 + 3.0 * std::sqrt(5.0)) / 20.0, b = (5.0 - std::sqrt(5.0)) / 20.0;
    const double pts[4][3] = {{b, b, b}, {a, b, b}, {b, a, b}, {b, b, a}};
    for (int q = 0; q < 4; ++q) {
      r.w.push_back(1.0 / 24.0);
      const double x = pts[q][0], y = pts[q][1], z = pts[q][2], l = 1 - x - y - z;
      // vertices 0..3, edges 4:(0,1) 5:(1,2) 6:(0,2) 7:(0,3) 8:(1,3) 9:(2,3)
      const double Lb[4] = {l, x, y, z};
      const double dL[4][3] = {{-1, -1, -1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
      const int ed[6][2] = {{0, 1}, {1, 2}, {0, 2}, {0, 3}, {1, 3}, {2, 3}};
      for (int v = 0; v < 4; ++v) {
        r.N.push_back(Lb[v] * (2 * Lb[v] - 1));
        for (int k = 0; k < 3; ++k) r.dN.push_back((4 * Lb[v] - 1) * dL[v][k]);
      }
      for (int e = 0; e < 6; ++e) {
        const int i = ed[e][0], j = ed[e][1];
        r.N.push_back(4 * Lb[i] * Lb[j]);
        for (int k = 0; k < 3; ++k) r.dN.push_back(4 * (dL[i][k] * Lb[j] + Lb[i] * dL[j][k]));
      }
    }
  } else if (et == ET_HEX27) {
    // triquadratic, 3x3x3 Gauss; node (i,j,k) index = i + 3j + 9k with 1D local order (-1, 0, 1)
    r.dim = 3; r.nnpe = 27; r.nq = 27;
    const double p3 = std::sqrt(0.6);
    const double gp[3] = {-p3, 0.0, p3}, gw[3] = {5.0 / 9.0, 8.0 / 9.0, 5.0 / 9.0};
    for (int qz = 0; qz < 3; ++qz)
      for (int qy = 0; qy < 3; ++qy)
        for (int qx = 0; qx < 3; ++qx) {
          r.w.push_back(gw[qx] * gw[qy] * gw[qz]);
          double vx[3], dx[3], vy[3], dy[3], vz[3], dz[3];
          lag2(gp[qx], vx, dx); lag2(gp[qy], vy, dy); lag2(gp[qz], vz, dz);
          for (int k = 0; k < 3; ++k)
            for (int j = 0; j < 3; ++j)
              for (int i = 0; i < 3; ++i) {
                r.N.push_back(vx[i] * vy[j] * vz[k]);
                r.dN.push_back(dx[i] * vy[j] * vz[k]);
                r.dN.push_back(vx[i] * dy[j] * vz[k]);
                r.dN.push_back(vx[i] * vy[j] * dz[k]);
              }
        }
  }
  return r;
}

// Caller-supplied tables (the ReferenceFE a caller builds with its own
// quadrature rule, src/FunctionSpaces.jl:104-126), set by orc_set_reference;
// otherwise the element type's default tables above.  Not for concurrent use
// with a change of tables.
RefFE g_override[9];
bool g_has_override[9] = {false};

const RefFE& ref_of(int et) {
  static thread_local RefFE defaults[9];
  if (et < 1 || et > 8) return defaults[0];
  if (g_has_override[et]) return g_override[et];
  if (defaults[et].nnpe == 0) defaults[et] = make_ref(et);
  return defaults[et];
}

struct Mapped {
  double JxW;
  double Xq[3];
  double dNX[27][3];
};

// J = X_el * dN_xi, JxW = det(J) w, dN_X = dN_xi * inv(J)
void map_qp(const RefFE& r, int q, const double* xel /*[a][d]*/, Mapped& m) {
  const int D = r.dim, A = r.nnpe;
  double J[3][3] = {{0}};
  for (int d = 0; d < D; ++d)
    for (int k = 0; k < D; ++k) {
      double s = 0;
      for (int a = 0; a < A; ++a) s += xel[a * D + d] * r.dN[(q * A + a) * D + k];
      J[d][k] = s;
    }
  double Ji[3][3] = {{0}};
  double det;
  if (D == 2) {
    det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
    Ji[0][0] = J[1][1] / det; Ji[0][1] = -J[0][1] / det;
    Ji[1][0] = -J[1][0] / det; Ji[1][1] = J[0][0] / det;
  } else {
    det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) - J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
          J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
    Ji[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / det;
    Ji[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;
    Ji[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
    Ji[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) / det;
    Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
    Ji[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;
    Ji[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / det;
    Ji[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;
    Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
  }
  m.JxW = det * r.w[q];
  for (int d = 0; d < 3; ++d) m.Xq[d] = 0;
  for (int d = 0; d < D; ++d) {
    double s = 0;
    for (int a = 0; a < A; ++a) s += r.N[q * A + a] * xel[a * D + d];
    m.Xq[d] = s;
  }
  for (int a = 0; a < A; ++a)
    for (int d = 0; d < D; ++d) {
      double s = 0;
      for (int k = 0; k < D; ++k) s += r.dN[(q * A + a) * D + k] * Ji[k][d];
      m.dNX[a][d] = s;
    }
}

// ---------------------------------------------------------------------------
// Physics
// ---------------------------------------------------------------------------
enum { PHYS_POISSON = 1, PHYS_NEOHOOKEAN = 2, PHYS_J2 = 3 };

// Poisson source f(X) = amp * prod_d sin(pi X_d)   (props[0] = amp)
inline double poisson_source(const double* X, int D, double amp) {
  double f = amp;
  for (int d = 0; d < D; ++d) f *= std::sin(M_PI * X[d]);
  return f;
}

// Neo-Hookean (TestMechanicsLargeDeformation.jl:17-27):
//   psi = K/2 (1/2 (J-1)^2 - ln J) + G/2 (J^{-2/3} tr(F F^T) - 3)
// P = dpsi/dF and A = d2psi/dF2 written out:  with H = F^{-T}, I1 = F:F,
//   P = c1 H + c2 (F - I1/3 H),  c1 = K/2 (J^2 - J - 1),  c2 = G J^{-2/3}
//   A_iJkL = (K/2 (2J-1) J + 2/9 c2 I1) H_iJ H_kL + (I1/3 c2 - c1) H_iL H_kJ
//            + c2 d_ik d_JL - 2/3 c2 (H_kL F_iJ + F_kL H_iJ)
// P9[i + 3J], A81[(i + 3J) + 9 (k + 3L)] (Tensors.jl column-major flattening).
void neohookean_PA(const double F[3][3], double Kb, double Gs, double* P9, double* A81) {
  const double J = F[0][0] * (F[1][1] * F[2][2] - F[1][2] * F[2][1]) - F[0][1] * (F[1][0] * F[2][2] - F[1][2] * F[2][0]) +
                   F[0][2] * (F[1][0] * F[2][1] - F[1][1] * F[2][0]);
  double H[3][3];  // F^{-T}: H[i][J] = cof(F)[i][J] / det
  H[0][0] = (F[1][1] * F[2][2] - F[1][2] * F[2][1]) / J;
  H[0][1] = (F[1][2] * F[2][0] - F[1][0] * F[2][2]) / J;
  H[0][2] = (F[1][0] * F[2][1] - F[1][1] * F[2][0]) / J;
  H[1][0] = (F[0][2] * F[2][1] - F[0][1] * F[2][2]) / J;
  H[1][1] = (F[0][0] * F[2][2] - F[0][2] * F[2][0]) / J;
  H[1][2] = (F[0][1] * F[2][0] - F[0][0] * F[2][1]) / J;
  H[2][0] = (F[0][1] * F[1][2] - F[0][2] * F[1][1]) / J;
  H[2][1] = (F[0][2] * F[1][0] - F[0][0] * F[1][2]) / J;
  H[2][2] = (F[0][0] * F[1][1] - F[0][1] * F[1][0]) / J;
  double I1 = 0;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) I1 += F[i][j] * F[i][j];
  const double c1 = 0.5 * Kb * (J * J - J - 1.0);
  const double c2 = Gs * std::pow(J, -2.0 / 3.0);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) P9[i + 3 * j] = c1 * H[i][j] + c2 * (F[i][j] - I1 / 3.0 * H[i][j]);
  if (!A81) return;
  const double a1 = 0.5 * Kb * (2.0 * J - 1.0) * J + 2.0 / 9.0 * c2 * I1;
  const double a2 = I1 / 3.0 * c2 - c1;
  for (int L = 0; L < 3; ++L)
    for (int k = 0; k < 3; ++k)
      for (int Jj = 0; Jj < 3; ++Jj)
        for (int i = 0; i < 3; ++i) {
          double v = a1 * H[i][Jj] * H[k][L] + a2 * H[i][L] * H[k][Jj] -
                     2.0 / 3.0 * c2 * (H[k][L] * F[i][Jj] + F[k][L] * H[i][Jj]);
          if (i == k && Jj == L) v += c2;
          A81[(i + 3 * Jj) + 9 * (k + 3 * L)] = v;
        }
}

// J2 small-strain plasticity, linear isotropic hardening, radial return
// (Simo & Hughes 1998, Box 3.2).  props: E, nu, sigma_y, H.  State (7):
// plastic strain eps_p (xx, yy, zz, yz, xz, xy tensor components) + eqps.
// Outputs the Cauchy stress as P9 (small strain: P = sigma) and the
// consistent tangent as A81 (major + minor symmetric).
void j2_update(const double gradu[3][3], const double* props, const double* st_old, double* st_new, double* P9,
               double* A81) {
  const double E = props[0], nu = props[1], sy = props[2], Hh = props[3];
  const double mu = E / (2 * (1 + nu)), lam = E * nu / ((1 + nu) * (1 - 2 * nu)), kap = lam + 2.0 / 3.0 * mu;
  double eps[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) eps[i][j] = 0.5 * (gradu[i][j] + gradu[j][i]);
  double ep[3][3] = {{st_old[0], st_old[5], st_old[4]}, {st_old[5], st_old[1], st_old[3]}, {st_old[4], st_old[3], st_old[2]}};
  const double eqps_old = st_old[6];
  double ee[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) ee[i][j] = eps[i][j] - ep[i][j];
  const double tr = ee[0][0] + ee[1][1] + ee[2][2];
  double s[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) s[i][j] = 2 * mu * (ee[i][j] - (i == j ? tr / 3.0 : 0.0));
  double snorm2 = 0;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) snorm2 += s[i][j] * s[i][j];
  const double snorm = std::sqrt(snorm2);
  const double sq23 = std::sqrt(2.0 / 3.0);
  const double f = snorm - sq23 * (sy + Hh * eqps_old);
  double n[3][3] = {{0}};
  double dgam = 0;
  if (f > 0) {
    dgam = f / (2 * mu + 2.0 / 3.0 * Hh);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) n[i][j] = s[i][j] / snorm;
  }
  double sig[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) sig[i][j] = s[i][j] - 2 * mu * dgam * n[i][j] + (i == j ? kap * tr : 0.0);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) P9[i + 3 * j] = sig[i][j];
  if (st_new) {
    double epn[3][3];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) epn[i][j] = ep[i][j] + dgam * n[i][j];
    st_new[0] = epn[0][0]; st_new[1] = epn[1][1]; st_new[2] = epn[2][2];
    st_new[3] = epn[1][2]; st_new[4] = epn[0][2]; st_new[5] = epn[0][1];
    st_new[6] = eqps_old + sq23 * dgam;
  }
  if (!A81) return;
  double th = 1.0, thb = 0.0;
  if (f > 0) {
    th = 1.0 - 2 * mu * dgam / snorm;
    thb = 1.0 / (1.0 + Hh / (3 * mu)) - (1.0 - th);
  }
  // C_ijkl = kap d_ij d_kl + 2 mu th (I_sym - 1/3 d_ij d_kl) - 2 mu thb n_ij n_kl
  for (int L = 0; L < 3; ++L)
    for (int k = 0; k < 3; ++k)
      for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i) {
          const double dij = i == j, dkl = k == L;
          const double Isym = 0.5 * ((i == k) * (j == L) + (i == L) * (j == k));
          A81[(i + 3 * j) + 9 * (k + 3 * L)] =
              kap * dij * dkl + 2 * mu * th * (Isym - dij * dkl / 3.0) - 2 * mu * thb * n[i][j] * n[k][L];
        }
}

}  // namespace

extern "C" {

// One element's residual and tangent, summed over quadrature points in q order
// (Assemblers.jl:418-431).  xel [a][d], uel [a][f], state arrays [q][s].
// Re[NDOF]; Ke[NDOF*NDOF] column-major like StaticArrays' K_el.data:
// Ke[r + NDOF*c] = dR_r / du_c.  Either output may be null.
// When set (per thread, by orc_assemble), orc_element also accumulates into it,
// per element dof, the magnitude of the terms its residual entry is formed
// from, down to the nodal values: sum_q JxW |grad N_a| (|grad u| + sum_b |u_b
// grad N_b|) + |N_a f| for Poisson, sum_q JxW |grad N_a|_1 (|P|_F + |A|_F |sum_b
// u_b (x) grad N_b|_F) for mechanics -- so that c eps times it bounds the
// rounding of any FP64 evaluation of the entry from the same nodal values.
thread_local double* tl_elem_abs = nullptr;

int orc_element(int et, int phys, const double* props, const double* xel, const double* uel,
                const double* st_old, double* st_new, double* Re, double* Ke) {
  if (et < 1 || et > 8) return -1;
  const RefFE& r = ref_of(et);
  if (r.nnpe == 0) return -1;
  const int D = r.dim, A = r.nnpe;
  const int NF = phys == PHYS_POISSON ? 1 : 3;
  if (phys != PHYS_POISSON && D != 3) return -2;
  const int NDOF = NF * A;
  if (Re) for (int i = 0; i < NDOF; ++i) Re[i] = 0;
  if (Ke) for (int i = 0; i < NDOF * NDOF; ++i) Ke[i] = 0;
  Mapped m;
  for (int q = 0; q < r.nq; ++q) {
    map_qp(r, q, xel, m);
    if (phys == PHYS_POISSON) {
      // R_q = grad u * dNX' - N' f(X_q);  K_q = dNX dNX'   (TestPoissonCommon.jl:75-107)
      double gu[3] = {0, 0, 0};
      for (int d = 0; d < D; ++d)
        for (int a = 0; a < A; ++a) gu[d] += uel[a] * m.dNX[a][d];
      const double f = poisson_source(m.Xq, D, props[0]);
      if (Re)
        for (int a = 0; a < A; ++a) {
          double s = 0;
          for (int d = 0; d < D; ++d) s += gu[d] * m.dNX[a][d];
          Re[a] += m.JxW * (s - r.N[q * A + a] * f);
          if (tl_elem_abs) {  // |grad u| and the sum of nodal terms it is formed from
            double sa = 0;
            for (int d = 0; d < D; ++d) {
              double g = 0;
              for (int b = 0; b < A; ++b) g += std::fabs(uel[b] * m.dNX[b][d]);
              sa += std::fabs(m.dNX[a][d]) * (std::fabs(gu[d]) + g);
            }
            tl_elem_abs[a] += std::fabs(m.JxW) * (sa + std::fabs(r.N[q * A + a] * f));
          }
        }
      if (Ke)
        for (int b = 0; b < A; ++b)
          for (int a = 0; a < A; ++a) {
            double s = 0;
            for (int d = 0; d < D; ++d) s += m.dNX[a][d] * m.dNX[b][d];
            Ke[a + NDOF * b] += m.JxW * s;
          }
    } else {
      double gu[3][3] = {{0}};
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
          for (int a = 0; a < A; ++a) gu[i][j] += uel[a * 3 + i] * m.dNX[a][j];
      double P9[9], A81[81];
      if (phys == PHYS_NEOHOOKEAN) {
        double F[3][3];
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j) F[i][j] = gu[i][j] + (i == j ? 1.0 : 0.0);
        neohookean_PA(F, props[0], props[1], P9, (Ke || tl_elem_abs) ? A81 : nullptr);
      } else if (phys == PHYS_J2) {
        j2_update(gu, props, st_old + 7 * q, st_new ? st_new + 7 * q : nullptr, P9,
                  (Ke || tl_elem_abs) ? A81 : nullptr);
      } else {
        return -3;
      }
      // f = G P, K = G A G^T with G[(a,i),(i,J)] = dNX[a][J]  (Formulations.jl:462-496)
      if (Re)
        for (int a = 0; a < A; ++a)
          for (int i = 0; i < 3; ++i) {
            double s = 0;
            for (int J = 0; J < 3; ++J) s += m.dNX[a][J] * P9[i + 3 * J];
            Re[a * 3 + i] += m.JxW * s;
          }
      if (Re && tl_elem_abs) {
        // |P| plus the stress the rounding of grad u can move: grad u is a sum of
        // nodal terms u_a (x) grad N_a much larger than itself where u is large
        // against its variation over an element (u ~ eps x cancels by ~x/h), and
        // |A| |that sum| bounds the resulting change of P
        double pn = 0, an = 0, gn = 0;
        for (int k = 0; k < 9; ++k) pn += P9[k] * P9[k];
        for (int k = 0; k < 81; ++k) an += A81[k] * A81[k];
        for (int i = 0; i < 3; ++i)
          for (int j = 0; j < 3; ++j) {
            double g = 0;
            for (int a = 0; a < A; ++a) g += std::fabs(uel[a * 3 + i] * m.dNX[a][j]);
            gn += g * g;
          }
        pn = std::sqrt(pn) + std::sqrt(an) * std::sqrt(gn);
        for (int a = 0; a < A; ++a) {
          const double g1 = std::fabs(m.dNX[a][0]) + std::fabs(m.dNX[a][1]) + std::fabs(m.dNX[a][2]);
          for (int i = 0; i < 3; ++i) tl_elem_abs[a * 3 + i] += std::fabs(m.JxW) * g1 * pn;
        }
      }
      if (Ke)
        for (int b = 0; b < A; ++b)
          for (int k = 0; k < 3; ++k)
            for (int a = 0; a < A; ++a)
              for (int i = 0; i < 3; ++i) {
                double s = 0;
                for (int J = 0; J < 3; ++J)
                  for (int L = 0; L < 3; ++L) s += m.dNX[a][J] * A81[(i + 3 * J) + 9 * (k + 3 * L)] * m.dNX[b][L];
                Ke[(a * 3 + i) + NDOF * (b * 3 + k)] += m.JxW * s;
              }
    }
  }
  return 0;
}

double* g_abs_out = nullptr;  // optional per-dof sums of |R_e| (orc_set_abs_output)

// The block loop of assemble_vector!/assemble_matrix! (Assemblers.jl:402-432).
//   R_full: length NF*NN, zeroed here, filled by scatter-add in element order
//           (serial when threads == 1; with threads > 1 the element loop runs in
//           parallel and the scatter is an atomic add, the reference's threaded
//           CPU behaviour).
//   Kstore: element-ordered slot storage, NDOF^2 per element, K_el.data order.
//   state arrays: per block (NS, NQ, NE) column-major, blocks concatenated.
// Either output may be null.  Returns 0 or a negative error.
int orc_assemble(int nblocks, const int* elem_types, const i64* ne, const i64* conn, int dim, const double* coords,
                 int phys, const double* props, const double* U, const double* st_old, double* st_new, i64 nn,
                 double* R_full, double* Kstore, int threads) {
  const int NF = phys == PHYS_POISSON ? 1 : 3;
  const int NS = phys == PHYS_J2 ? 7 : 0;
  if (R_full)
    for (i64 i = 0; i < NF * nn; ++i) R_full[i] = 0;
  i64 coff = 0, koff = 0, soff = 0;
  int err = 0;
  double* R_abs = R_full ? g_abs_out : nullptr;
  if (R_abs)
    for (i64 i = 0; i < NF * nn; ++i) R_abs[i] = 0;
  for (int b = 0; b < nblocks; ++b) {
    const RefFE& r = ref_of(elem_types[b]);
    if (r.nnpe == 0 || r.dim != dim) return -1;
    const int A = r.nnpe, NDOF = NF * A;
    const i64 NEb = ne[b];
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(threads > 0 ? threads : 1) if (threads > 1)
#endif
    for (i64 e = 0; e < NEb; ++e) {
      const i64* c = conn + coff + e * A;
      double xel[27 * 3], uel[27 * 3], Re[81], Ke[81 * 81];
      for (int a = 0; a < A; ++a) {
        for (int d = 0; d < dim; ++d) xel[a * dim + d] = coords[(c[a] - 1) * dim + d];
        for (int f = 0; f < NF; ++f) uel[a * NF + f] = U[(c[a] - 1) * NF + f];
      }
      const double* so = NS ? st_old + soff + e * NS * r.nq : nullptr;
      double* sn = (NS && st_new) ? st_new + soff + e * NS * r.nq : nullptr;
      double so_zero[7 * 27] = {0};
      double Rabs[81] = {0};
      tl_elem_abs = R_abs ? Rabs : nullptr;
      int rc = orc_element(elem_types[b], phys, props, xel, uel, so ? so : so_zero, sn, R_full ? Re : nullptr,
                           Kstore ? Ke : nullptr);
      tl_elem_abs = nullptr;
      if (rc) err = rc;
      if (R_full) {
        for (int f = 0; f < NF; ++f)
          for (int a = 0; a < A; ++a) {
            double* dst = &R_full[NF * (c[a] - 1) + f];
            const double v = Re[NF * a + f];
            if (threads > 1) {
#ifdef _OPENMP
#pragma omp atomic
#endif
              *dst += v;
            } else {
              *dst += v;
            }
            if (R_abs) {
              double* da = &R_abs[NF * (c[a] - 1) + f];
#ifdef _OPENMP
#pragma omp atomic
#endif
              *da += Rabs[NF * a + f];
            }
          }
      }
      if (Kstore) std::memcpy(Kstore + koff + e * NDOF * NDOF, Ke, sizeof(double) * NDOF * NDOF);
    }
    coff += NEb * A;
    koff += NEb * NDOF * NDOF;
    soff += NEb * NS * r.nq;
  }
  return err;
}

// With a non-null `out` (NF * NN doubles), the next orc_assemble calls with a
// residual also write out[dof] = the sum over the dof's elements of the
// magnitudes of the terms its residual entry sums (see tl_elem_abs): the scale
// against which the rounding of an assembled residual entry is measured, whose
// value results from cancelling sums (of element forces near equilibrium, and
// inside the stress itself).  NULL turns it off.
void orc_set_abs_output(double* out) { g_abs_out = out; }

// Quadrature-point count of an element type (0 if unknown).
int orc_num_qp(int et) { return ref_of(et).nq; }

// Installs caller tables for element type et (N [nq][nnpe], dN [nq][nnpe][dim],
// w [nq]); nq may be 1..27.  orc_clear_reference(et) restores the
// defaults.  Returns 0 or -1 for an unknown element type.
int orc_set_reference(int et, int nq, const double* N, const double* dN, const double* w) {
  if (et < 1 || et > 8 || nq <= 0 || nq > 27) return -1;
  const RefFE d = make_ref(et);
  if (d.nnpe == 0) return -1;
  RefFE r;
  r.dim = d.dim;
  r.nnpe = d.nnpe;
  r.nq = nq;
  r.N.assign(N, N + size_t(nq) * d.nnpe);
  r.dN.assign(dN, dN + size_t(nq) * d.nnpe * d.dim);
  r.w.assign(w, w + nq);
  g_override[et] = r;
  g_has_override[et] = true;
  return 0;
}

void orc_clear_reference(int et) {
  if (et >= 1 && et <= 8) g_has_override[et] = false;
}

// Neo-Hookean P and A at one deformation gradient (F row-major [i][J]).
void orc_neohookean_PA(const double* F9, double Kb, double Gs, double* P9, double* A81) {
  double F[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) F[i][j] = F9[3 * i + j];
  neohookean_PA(F, Kb, Gs, P9, A81);
}

// J2 update at one point (gradu row-major [i][j]).
void orc_j2_update(const double* gu9, const double* props, const double* st_old, double* st_new, double* P9,
                   double* A81) {
  double gu[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) gu[i][j] = gu9[3 * i + j];
  j2_update(gu, props, st_old, st_new, P9, A81);
}

int orc_max_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"
