// Host-side set-up of a finite-elasticity equations set (libcm_fe).
//
// Runs once per handle and produces the device-resident index data:
//   * dof numbering — separated-component order of the reference's dependent
//     field on one rank (field_routines.f90:10330-10540);
//   * the CSR sparsity pattern, following the rule of
//     JacobianMatrix_StructureCalculate (equations_matrices_routines.f90:
//     5085-5300): a row's columns are every dof of every component of every
//     element around the row's node (or of the row's own element for an
//     element-based pressure), sorted and de-duplicated.  Because dofs are
//     component-major, each row is [u_x block | u_y block | u_z block | p
//     block] with the three u blocks holding the same sorted node set, which
//     is what the rank tables below exploit;
//   * an element colouring (no two elements of one colour share a node), so
//     that the device scatter is race-free and deterministic;
//   * per element, the position of every (row node, column node) pair inside
//     the CSR rows ("rank") plus a bit telling whether the element is the first
//     one — in colour order — to touch that CSR slot.  First contributors
//     store, later ones add, so no pass zeroes the matrix.  Identical tables
//     are shared between elements;
//   * the geometric Gauss-point data: dXi/dNu and the volume Jacobian J_x,
//     computed with the same formulas the reference re-evaluates at every
//     Gauss point of every evaluation (COORDINATE_METRICS_CALCULATE,
//     coordinate_routines.f90:647-833; Coordinates_MaterialSystemCalculate,
//     :3883-4149).  The geometry does not change during a solve, so it is
//     computed here once.
#include <algorithm>
#include <array>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <thread>
#include <unordered_map>

#include "fe_internal.h"

namespace cmfe {
namespace {

const double ZERO_TOL = 5.0 * DBL_EPSILON;  // ZERO_TOLERANCE, constants.f90:68

// 1-D Lagrange basis values/derivatives (basis_routines.f90:7015-7130).
double lag1d(int nodes, int k, int d, double t) {
  if (nodes == 2) {
    if (d == 0) return k == 0 ? 1.0 - t : t;
    return k == 0 ? -1.0 : 1.0;
  }
  if (d == 0) {
    if (k == 0) return 1.0 - 3.0 * t + 2.0 * t * t;
    if (k == 1) return 4.0 * t * (1.0 - t);
    return t * (t + t - 1.0);
  }
  if (k == 0) return 4.0 * t - 3.0;
  if (k == 1) return 4.0 - 8.0 * t;
  return 4.0 * t - 1.0;
}

// Tensor-product Lagrange tables on the 3-point Gauss-Legendre rule over
// [0,1]^3 (GAUSS_LEGENDRE basis_routines.f90:5840-5868; point ng = i+3j+9k,
// weight w_i w_j w_k, :2860-2872).  Layout gbf[g][d][a], d = value, d/dxi1..3.
void quad_tables(int n1, std::vector<double>& gbf, std::vector<double>& w) {
  const double pt[3] = {(-std::sqrt(0.6) + 1.0) / 2.0, 0.5, (std::sqrt(0.6) + 1.0) / 2.0};
  const double wt[3] = {2.5 / 9.0, 4.0 / 9.0, 2.5 / 9.0};
  const int nn = n1 * n1 * n1;
  gbf.assign((size_t)NG * 4 * nn, 0.0);
  w.assign(NG, 0.0);
  for (int k = 0; k < 3; ++k)
    for (int j = 0; j < 3; ++j)
      for (int i = 0; i < 3; ++i) {
        const int g = i + 3 * j + 9 * k;
        w[g] = wt[i] * wt[j] * wt[k];
        const double xi[3] = {pt[i], pt[j], pt[k]};
        for (int a = 0; a < nn; ++a) {
          const int pos[3] = {a % n1, (a / n1) % n1, a / (n1 * n1)};
          for (int d = 0; d < 4; ++d) {
            double v = 1.0;
            for (int c = 0; c < 3; ++c) v = v * lag1d(n1, pos[c], (d == c + 1) ? 1 : 0, xi[c]);
            gbf[((size_t)g * 4 + d) * nn + a] = v;
          }
        }
      }
}

// 3x3 inverse by cofactors with the determinant (INVERT_FULL_DP, maths.f90:1484-1498).
double inv3(const double a[3][3], double b[3][3]) {
  const double det = a[0][0] * a[1][1] * a[2][2] + a[0][1] * a[1][2] * a[2][0] + a[0][2] * a[1][0] * a[2][1] -
                     a[0][0] * a[2][1] * a[1][2] - a[1][0] * a[0][1] * a[2][2] - a[2][0] * a[1][1] * a[0][2];
  if (std::fabs(det) > ZERO_TOL) {
    b[0][0] = (a[1][1] * a[2][2] - a[2][1] * a[1][2]) / det;
    b[1][0] = (a[1][2] * a[2][0] - a[2][2] * a[1][0]) / det;
    b[2][0] = (a[1][0] * a[2][1] - a[2][0] * a[1][1]) / det;
    b[0][1] = (a[2][1] * a[0][2] - a[0][1] * a[2][2]) / det;
    b[1][1] = (a[2][2] * a[0][0] - a[0][2] * a[2][0]) / det;
    b[2][1] = (a[2][0] * a[0][1] - a[0][0] * a[2][1]) / det;
    b[0][2] = (a[0][1] * a[1][2] - a[1][1] * a[0][2]) / det;
    b[1][2] = (a[0][2] * a[1][0] - a[1][2] * a[0][0]) / det;
    b[2][2] = (a[0][0] * a[1][1] - a[1][0] * a[0][1]) / det;
  } else {
    std::memset(b, 0, sizeof(double) * 9);
  }
  return det;
}

void mul3(const double a[3][3], const double b[3][3], double c[3][3]) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) c[i][j] = a[i][0] * b[0][j] + a[i][1] * b[1][j] + a[i][2] * b[2][j];
}

void unit3(const double a[3], double o[3]) {
  double s = 0.0;
  for (int i = 0; i < 3; ++i) s = s + a[i] * a[i];
  const double l = std::sqrt(s);
  for (int i = 0; i < 3; ++i) o[i] = (std::fabs(l) < ZERO_TOL) ? a[i] : a[i] / l;
}

// dXi/dNu of the material frame: the reference frame built from dX/dxi1 and
// dX/dxi2, rotated by the fibre, imbrication and sheet angles
// (coordinate_routines.f90:4042-4149), or dXi/dX without fibres (:3929-3940).
void dxi_dnu(const double dxdxi[3][3], const double* ang, double out[3][3]) {
  double m[3][3];
  if (ang) {
    const double f[3] = {dxdxi[0][0], dxdxi[1][0], dxdxi[2][0]};
    const double f2[3] = {dxdxi[0][1], dxdxi[1][1], dxdxi[2][1]};
    double h[3] = {f[1] * f2[2] - f[2] * f2[1], f[2] * f2[0] - f[0] * f2[2], f[0] * f2[1] - f[1] * f2[0]};
    double g[3] = {h[1] * f[2] - h[2] * f[1], h[2] * f[0] - h[0] * f[2], h[0] * f[1] - h[1] * f[0]};
    double nf[3], ng[3], nh[3];
    unit3(f, nf);
    unit3(g, ng);
    unit3(h, nh);
    double R[3][3] = {{nf[0], ng[0], nh[0]}, {nf[1], ng[1], nh[1]}, {nf[2], ng[2], nh[2]}};
    double ca = std::cos(ang[0]), sa = std::sin(ang[0]);
    double cb = std::cos(ang[1]), sb = std::sin(ang[1]);
    double cg = std::cos(ang[2]), sg = std::sin(ang[2]);
    double Ra[3][3] = {{ca, -1.0 * sa, 0.0}, {sa, ca, 0.0}, {0.0, 0.0, 1.0}};
    double Rb[3][3] = {{cb, 0.0, sb}, {0.0, 1.0, 0.0}, {-1.0 * sb, 0.0, cb}};
    double Rc[3][3] = {{1.0, 0.0, 0.0}, {0.0, cg, -1.0 * sg}, {0.0, sg, cg}};
    double t1[3][3], t2[3][3], dxdnu[3][3], dnudx[3][3];
    mul3(R, Ra, t1);
    mul3(t1, Rb, t2);
    mul3(t2, Rc, dxdnu);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) dnudx[i][j] = dxdnu[j][i];
    mul3(dnudx, dxdxi, m);
  } else {
    std::memcpy(m, dxdxi, sizeof(m));
  }
  inv3(m, out);
}

int fail(std::string& msg, const std::string& what) {
  msg = what;
  return FE_ERR_INVALID_ARGUMENT;
}

// Sorted, de-duplicated union.
void sort_unique(std::vector<int32_t>& v) {
  std::sort(v.begin(), v.end());
  v.erase(std::unique(v.begin(), v.end()), v.end());
}

template <class F>
void parallel_for(int n, F f) {
  // one thread per 1,024 items at most (thread start-up outweighs smaller shares)
  unsigned nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  nt = std::max(1u, std::min(nt, (unsigned)(n / 1024)));
  if (nt == 1) {
    for (int i = 0; i < n; ++i) f(i);
    return;
  }
  std::vector<std::thread> th;
  const int chunk = (n + (int)nt - 1) / (int)nt;
  for (unsigned t = 0; t < nt; ++t)
    th.emplace_back([&, t]() {
      const int lo = (int)t * chunk, hi = std::min(n, lo + chunk);
      for (int i = lo; i < hi; ++i) f(i);
    });
  for (auto& x : th) x.join();
}

}  // namespace

int build_setup(const fe_mesh_desc* d, HostSetup& s, std::string& msg) {
  if (!d) return fail(msg, "mesh description is NULL");
  if (d->num_elements <= 0 || d->num_nodes_u <= 0) return fail(msg, "mesh has no elements or nodes");
  if (d->nodes_per_xi_u != 2 && d->nodes_per_xi_u != 3)
    return fail(msg, "nodes_per_xi_u must be 2 (trilinear) or 3 (triquadratic)");
  if (d->pressure_interpolation != FE_PRESSURE_ELEMENT_BASED && d->pressure_interpolation != FE_PRESSURE_NODE_BASED)
    return fail(msg, "invalid pressure interpolation");
  if (d->law != FE_LAW_MOONEY_RIVLIN && d->law != FE_LAW_GUCCIONE)
    return fail(msg, "law must be FE_LAW_MOONEY_RIVLIN or FE_LAW_GUCCIONE");
  const int need_mat = d->law == FE_LAW_MOONEY_RIVLIN ? 2 : 4;
  if (d->num_material_components != need_mat) return fail(msg, "wrong number of material components for the law");
  if (!d->element_nodes_u || !d->geometry || !d->materials) return fail(msg, "NULL mesh array");
  if (d->pressure_interpolation == FE_PRESSURE_NODE_BASED && (!d->element_nodes_p || d->num_nodes_p <= 0))
    return fail(msg, "node-based pressure needs element_nodes_p and num_nodes_p");

  s.ne = d->num_elements;
  s.nu = d->num_nodes_u;
  s.n1 = d->nodes_per_xi_u;
  s.npe = s.n1 * s.n1 * s.n1;
  s.pmode = d->pressure_interpolation;
  s.npp = s.pmode ? 8 : 1;
  s.npn = s.pmode ? d->num_nodes_p : s.ne;
  s.nr = s.npe + s.npp;
  s.nrow = 3 * s.npe + s.npp;
  s.law = d->law;
  s.nmat = need_mat;
  s.mat_per_element = d->materials_per_element ? 1 : 0;
  s.fibre = d->fibre_angles != nullptr;
  s.ndofs = 3ll * s.nu + s.npn;
  if (s.ndofs >= (1ll << 31)) return fail(msg, "too many dofs for 32-bit CSR indices");

  s.elem_u.assign(d->element_nodes_u, d->element_nodes_u + (size_t)s.ne * s.npe);
  for (int32_t v : s.elem_u)
    if (v < 0 || v >= s.nu) return fail(msg, "element_nodes_u entry out of range");
  if (s.pmode) {
    s.elem_p.assign(d->element_nodes_p, d->element_nodes_p + (size_t)s.ne * 8);
    for (int32_t v : s.elem_p)
      if (v < 0 || v >= s.npn) return fail(msg, "element_nodes_p entry out of range");
  }
  s.mat.assign(d->materials, d->materials + (size_t)s.nmat * (s.mat_per_element ? s.ne : 1));

  // Element -> row-node accessors: local row node r < npe is a u node, else a
  // pressure row node (pressure node, or the element itself when element-based).
  auto unode = [&](int e, int a) { return s.elem_u[(size_t)e * s.npe + a]; };
  auto pnode = [&](int e, int q) { return s.pmode ? s.elem_p[(size_t)e * 8 + q] : e; };

  // Elements around each u node and each pressure row node.
  std::vector<std::vector<int32_t>> surr_u(s.nu), surr_p(s.npn);
  for (int e = 0; e < s.ne; ++e) {
    for (int a = 0; a < s.npe; ++a) surr_u[unode(e, a)].push_back(e);
    for (int q = 0; q < s.npp; ++q) surr_p[pnode(e, q)].push_back(e);
  }
  for (auto& v : surr_u) sort_unique(v);
  for (auto& v : surr_p) sort_unique(v);
  for (int n = 0; n < s.nu; ++n)
    if (surr_u[n].empty()) return fail(msg, "a u node belongs to no element");

  // Incidence lists of the staged assembly (elements in increasing order).
  s.u_inc_ptr.assign((size_t)s.nu + 1, 0);
  s.p_inc_ptr.assign((size_t)s.npn + 1, 0);
  for (int n = 0; n < s.nu; ++n) s.u_inc_ptr[n + 1] = s.u_inc_ptr[n] + (int32_t)surr_u[n].size();
  for (int q = 0; q < s.npn; ++q) s.p_inc_ptr[q + 1] = s.p_inc_ptr[q] + (int32_t)surr_p[q].size();
  s.u_inc.resize(s.u_inc_ptr[s.nu]);
  s.p_inc.resize(s.p_inc_ptr[s.npn]);
  if ((int64_t)s.ne * 32 >= (1ll << 31)) return fail(msg, "too many elements for the staged assembly's incidence lists");
  parallel_for(s.nu, [&](int n) {
    int32_t k = s.u_inc_ptr[n];
    for (int e : surr_u[n]) {
      int la = 0;
      while (unode(e, la) != n) ++la;
      s.u_inc[k++] = e * 32 + la;
    }
  });
  parallel_for(s.npn, [&](int q) {
    int32_t k = s.p_inc_ptr[q];
    for (int e : surr_p[q]) {
      int lq = 0;
      while (pnode(e, lq) != q) ++lq;
      s.p_inc[k++] = e * 8 + lq;
    }
  });

  // Completion order of the rows: the largest element around nodes 0..a.
  s.u_last_prefix.resize(s.nu);
  s.p_last_prefix.resize(s.npn);
  for (int n = 0, m = -1; n < s.nu; ++n) {
    if (!surr_u[n].empty()) m = std::max(m, surr_u[n].back());
    s.u_last_prefix[n] = m;
  }
  for (int q = 0, m = -1; q < s.npn; ++q) {
    if (!surr_p[q].empty()) m = std::max(m, surr_p[q].back());
    s.p_last_prefix[q] = m;
  }

  // Neighbourhoods: sorted u nodes and sorted pressure row nodes around every row node.
  std::vector<std::vector<int32_t>> nbu_u(s.nu), nbp_u(s.nu), nbu_p(s.npn), nbp_p(s.npn);
  auto fill_nb = [&](const std::vector<int32_t>& elems, std::vector<int32_t>& nu_out, std::vector<int32_t>& np_out) {
    // gathered in per-thread scratch, stored at their final size
    thread_local std::vector<int32_t> su, sp;
    su.clear();
    sp.clear();
    for (int e : elems) {
      for (int a = 0; a < s.npe; ++a) su.push_back(unode(e, a));
      for (int q = 0; q < s.npp; ++q) sp.push_back(pnode(e, q));
    }
    sort_unique(su);
    sort_unique(sp);
    nu_out.assign(su.begin(), su.end());
    np_out.assign(sp.begin(), sp.end());
  };
  parallel_for(s.nu, [&](int n) { fill_nb(surr_u[n], nbu_u[n], nbp_u[n]); });
  parallel_for(s.npn, [&](int q) { fill_nb(surr_p[q], nbu_p[q], nbp_p[q]); });

  s.wu.resize(s.nu);
  s.wp.resize(s.npn);
  for (int n = 0; n < s.nu; ++n) s.wu[n] = (int32_t)nbu_u[n].size();
  for (int q = 0; q < s.npn; ++q) s.wp[q] = (int32_t)nbu_p[q].size();

  // CSR pattern (0-based) and the mixed split.
  s.row_ptr.assign(s.ndofs + 1, 0);
  s.uu_row_ptr.assign(3ll * s.nu + 1, 0);
  s.cp_row_ptr.assign(s.ndofs + 1, 0);
  int64_t nnz = 0, nuu = 0, ncp = 0;
  for (int64_t r = 0; r < s.ndofs; ++r) {
    const bool urow = r < 3ll * s.nu;
    const int node = urow ? (int)(r % s.nu) : (int)(r - 3ll * s.nu);
    const int64_t wu_ = urow ? nbu_u[node].size() : nbu_p[node].size();
    const int64_t wp_ = urow ? nbp_u[node].size() : nbp_p[node].size();
    nnz += 3 * wu_ + wp_;
    if (urow) {
      nuu += 3 * wu_;
      ncp += wp_;
      s.uu_row_ptr[r + 1] = (int32_t)nuu;
    } else {
      ncp += 3 * wu_ + wp_;
    }
    if (nnz >= (1ll << 31) || ncp >= (1ll << 31)) return fail(msg, "too many nonzeros for 32-bit CSR indices");
    s.row_ptr[r + 1] = (int32_t)nnz;
    s.cp_row_ptr[r + 1] = (int32_t)ncp;
  }
  s.nnz = nnz;
  s.nnz_uu = nuu;
  s.nnz_cp = ncp;
  {
    // scratch of one gathering warp: the larger of a u node's three rows
    // (3 x 3 wu FP32, padded to 16 bytes, then 3 x its pressure columns FP64)
    // and a pressure row (FP64)
    int64_t need = 0;
    for (int n = 0; n < s.nu; ++n) {
      const int64_t wc = s.cp_row_ptr[(size_t)n + 1] - s.cp_row_ptr[(size_t)n];
      need = std::max<int64_t>(need, ((36 * (int64_t)s.wu[n] + 15) & ~(int64_t)15) + 3 * wc * 8);
    }
    for (int q = 0; q < s.npn; ++q) {
      const size_t row = (size_t)3 * s.nu + q;
      need = std::max<int64_t>(need, (int64_t)(s.cp_row_ptr[row + 1] - s.cp_row_ptr[row]) * 8);
    }
    s.gather_bytes = (int)std::min<int64_t>((need + 15) & ~(int64_t)15, 1 << 30);
  }


  s.col.allocate(nnz);
  parallel_for((int)s.ndofs, [&](int r) {
    const bool urow = r < 3ll * s.nu;
    const int node = urow ? (int)(r % s.nu) : (int)(r - 3ll * s.nu);
    const auto& U = urow ? nbu_u[node] : nbu_p[node];
    const auto& Pn = urow ? nbp_u[node] : nbp_p[node];
    int64_t k = s.row_ptr[r];
    for (int c = 0; c < 3; ++c)
      for (int32_t v : U) s.col[k++] = c * s.nu + v;
    for (int32_t v : Pn) s.col[k++] = (int32_t)(3ll * s.nu + v);
  });

  // Greedy colouring in element order: the smallest colour not used by an
  // element sharing any node (u or pressure).
  std::vector<int32_t> colour(s.ne, 0);
  s.ncolours = 0;
  {
    std::vector<char> used;
    for (int e = 0; e < s.ne; ++e) {
      used.assign(64, 0);
      for (int a = 0; a < s.npe; ++a)
        for (int f : surr_u[unode(e, a)])
          if (f < e) used[colour[f]] = 1;
      for (int q = 0; q < s.npp; ++q)
        for (int f : surr_p[pnode(e, q)])
          if (f < e) used[colour[f]] = 1;
      int c = 0;
      while (c < 64 && used[c]) ++c;
      if (c == 64) return fail(msg, "element colouring needs more than 64 colours");
      colour[e] = c;
      s.ncolours = std::max(s.ncolours, c + 1);
    }
  }
  s.colour_ptr.assign(s.ncolours + 1, 0);
  for (int e = 0; e < s.ne; ++e) s.colour_ptr[colour[e] + 1]++;
  for (int c = 0; c < s.ncolours; ++c) s.colour_ptr[c + 1] += s.colour_ptr[c];
  s.colour_elems.resize(s.ne);
  {
    std::vector<int32_t> fillp(s.colour_ptr.begin(), s.colour_ptr.end() - 1);
    for (int e = 0; e < s.ne; ++e) s.colour_elems[fillp[colour[e]]++] = e;
  }

  // Per-element rank / first-contributor tables.
  const int nr = s.nr;
  std::vector<uint16_t> etab((size_t)s.ne * nr * nr);
  std::vector<char> bad(s.ne, 0);
  parallel_for(s.ne, [&](int e) {
    uint16_t* T = &etab[(size_t)e * nr * nr];
    int32_t rn[64];
    bool isu[64];
    for (int a = 0; a < s.npe; ++a) { rn[a] = unode(e, a); isu[a] = true; }
    for (int q = 0; q < s.npp; ++q) { rn[s.npe + q] = pnode(e, q); isu[s.npe + q] = false; }
    // ranks: the column nodes of each kind in increasing order, merged with
    // each row node's sorted neighbour list of that kind
    int cols[2][64], ncol[2] = {0, 0};  // [u | p] local column indices, by increasing node number
    for (int cb = 0; cb < nr; ++cb) {
      const int k = isu[cb] ? 0 : 1;
      int i = ncol[k]++;
      while (i > 0 && rn[cols[k][i - 1]] > rn[cb]) {
        cols[k][i] = cols[k][i - 1];
        --i;
      }
      cols[k][i] = cb;
    }
    for (int ra = 0; ra < nr; ++ra)
      for (int k = 0; k < 2; ++k) {
        const std::vector<int32_t>& L = isu[ra] ? (k == 0 ? nbu_u[rn[ra]] : nbp_u[rn[ra]])
                                                : (k == 0 ? nbu_p[rn[ra]] : nbp_p[rn[ra]]);
        size_t j = 0;
        for (int i = 0; i < ncol[k]; ++i) {
          const int cb = cols[k][i];
          while (j < L.size() && L[j] < rn[cb]) ++j;
          if (j == L.size() || L[j] != rn[cb] || j > 0x7fff) { bad[e] = 1; return; }
          T[ra * nr + cb] = (uint16_t)j | 0x8000;
        }
      }
    // first-contributor bits: cleared where an element of a lower colour also
    // holds both the row node and the column node.
    thread_local std::vector<int32_t> nbe;  // reused: no allocation per element
    nbe.clear();
    for (int a = 0; a < s.npe; ++a)
      for (int f : surr_u[rn[a]]) nbe.push_back(f);
    for (int q = 0; q < s.npp; ++q)
      for (int f : surr_p[rn[s.npe + q]]) nbe.push_back(f);
    sort_unique(nbe);
    for (int f : nbe) {
      if (f == e || colour[f] >= colour[e]) continue;
      // the row nodes of e that f also holds (f is in the sorted list of
      // elements around each of them)
      int shared[64], ns = 0;
      for (int r = 0; r < nr; ++r) {
        const std::vector<int32_t>& around = isu[r] ? surr_u[rn[r]] : surr_p[rn[r]];
        if (std::binary_search(around.begin(), around.end(), f)) shared[ns++] = r;
      }
      for (int i = 0; i < ns; ++i)
        for (int j = 0; j < ns; ++j) T[shared[i] * nr + shared[j]] &= 0x7fff;
    }
  });
  for (int e = 0; e < s.ne; ++e)
    if (bad[e]) {
      msg = "internal error: element entry missing from the CSR pattern";
      return FE_ERR_PATTERN;
    }
  // share identical tables
  s.elem_table.resize(s.ne);
  {
    std::unordered_map<std::string, int> seen;
    const size_t bytes = (size_t)nr * nr * sizeof(uint16_t);
    for (int e = 0; e < s.ne; ++e) {
      std::string key((const char*)&etab[(size_t)e * nr * nr], bytes);
      auto it = seen.find(key);
      if (it == seen.end()) {
        int id = (int)seen.size();
        seen.emplace(std::move(key), id);
        s.tables.insert(s.tables.end(), &etab[(size_t)e * nr * nr], &etab[(size_t)e * nr * nr] + nr * nr);
        s.elem_table[e] = id;
      } else {
        s.elem_table[e] = it->second;
      }
    }
    s.ntables = (int)seen.size();
  }

  // Boundary faces: a local face (reference order -xi1, -xi2, -xi3, +xi1,
  // +xi2, +xi3) whose four corner nodes no other element holds.
  {
    auto corners = [&](int e, int lf, std::array<int32_t, 4>& c4) {
      const int ni = lf % 3, side = lf / 3, xa = ni == 0 ? 1 : 0, xb = ni == 2 ? 1 : 2, n1 = s.n1;
      int k = 0;
      for (int f2 = 0; f2 < 2; ++f2)
        for (int f1 = 0; f1 < 2; ++f1) {
          int pos[3];
          pos[ni] = side ? n1 - 1 : 0;
          pos[xa] = f1 ? n1 - 1 : 0;
          pos[xb] = f2 ? n1 - 1 : 0;
          c4[k++] = unode(e, pos[0] + n1 * (pos[1] + n1 * pos[2]));
        }
      std::sort(c4.begin(), c4.end());
    };
    // the sorted corner quadruple of every local face; a face is on the
    // boundary when no other (element, local face) pair has the same
    // quadruple -- every such pair holds the face's lowest corner, so only the
    // elements around that node are compared
    std::vector<std::array<int32_t, 4>> fc((size_t)s.ne * 6);
    parallel_for(s.ne, [&](int e) {
      for (int lf = 0; lf < 6; ++lf) corners(e, lf, fc[(size_t)e * 6 + lf]);
    });
    s.bnd_mask.assign(s.ne, 0);
    parallel_for(s.ne, [&](int e) {
      uint8_t mask = 0;
      for (int lf = 0; lf < 6; ++lf) {
        const auto& c4 = fc[(size_t)e * 6 + lf];
        int count = 0;
        for (int f : surr_u[c4[0]])
          for (int lg = 0; lg < 6; ++lg) count += fc[(size_t)f * 6 + lg] == c4;
        if (count == 1) mask |= (uint8_t)(1u << lf);
      }
      s.bnd_mask[e] = mask;
    });
    s.bnd_ptr.assign(s.ncolours + 1, 0);
    s.bnd_elems.clear();
    for (int c = 0; c < s.ncolours; ++c) {
      for (int i = s.colour_ptr[c]; i < s.colour_ptr[c + 1]; ++i)
        if (s.bnd_mask[s.colour_elems[i]]) s.bnd_elems.push_back(s.colour_elems[i]);
      s.bnd_ptr[c + 1] = (int32_t)s.bnd_elems.size();
    }
  }

  // Quadrature tables.
  quad_tables(s.n1, s.gbf_u, s.gw);
  {
    std::vector<double> g2, w2;
    quad_tables(2, g2, w2);
    s.gbf_p.assign((size_t)NG * 8, 0.0);
    for (int g = 0; g < NG; ++g)
      for (int q = 0; q < 8; ++q) s.gbf_p[(size_t)g * 8 + q] = g2[((size_t)g * 4 + 0) * 8 + q];
  }

  // Geometric Gauss-point data.
  s.geo.assign((size_t)s.ne * NG * 10, 0.0);
  std::vector<char> degenerate(s.ne, 0);
  parallel_for(s.ne, [&](int e) {
    for (int g = 0; g < NG; ++g) {
      double dxdxi[3][3], ang[3];
      for (int c = 0; c < 3; ++c) {
        for (int k = 0; k < 3; ++k) {
          double acc = 0.0;
          for (int a = 0; a < s.npe; ++a)
            acc = acc + s.gbf_u[((size_t)g * 4 + k + 1) * s.npe + a] * d->geometry[(size_t)c * s.nu + unode(e, a)];
          dxdxi[c][k] = acc;
        }
        if (s.fibre) {
          double acc = 0.0;
          for (int a = 0; a < s.npe; ++a)
            acc = acc + s.gbf_u[((size_t)g * 4) * s.npe + a] * d->fibre_angles[(size_t)c * s.nu + unode(e, a)];
          ang[c] = acc;
        }
      }
      double gl[3][3], gu[3][3], dn[3][3];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
          gl[i][j] = dxdxi[0][i] * dxdxi[0][j] + dxdxi[1][i] * dxdxi[1][j] + dxdxi[2][i] * dxdxi[2][j];
      const double det_gl = inv3(gl, gu);
      dxi_dnu(dxdxi, s.fibre ? ang : nullptr, dn);
      double* out = &s.geo[((size_t)e * NG + g) * 10];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) out[i * 3 + j] = dn[i][j];
      out[9] = std::sqrt(std::fabs(det_gl));
      if (!(out[9] > 0.0)) degenerate[e] = 1;
    }
  });
  for (int e = 0; e < s.ne; ++e)
    if (degenerate[e]) return fail(msg, "degenerate element geometry (zero volume Jacobian)");
  return FE_NO_ERROR;
}

}  // namespace cmfe
