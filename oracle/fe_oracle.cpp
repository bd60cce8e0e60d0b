// ============================================================================
// TEST INFRASTRUCTURE ONLY — the FP64 CPU oracle for finite-elasticity
// assembly.  Nothing in the shipped library links, loads or calls this file;
// only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg do, as
// the checker and as the timed CPU baseline.
//
// A plain C++ restatement of OpenCMISS-Iron's (OpenCMISS/cm) Fortran hot path
// for incompressible Mooney-Rivlin and transversely-isotropic Guccione
// finite elasticity, following the reference's formulas and loop order
// (1-based Fortran indices are written 0-based here).  The reference itself
// is Fortran 2003 + MPI + PETSc and cannot be compiled here (no gfortran, no
// MPI, no PETSc), so this restatement is the oracle.
//
// Parity pinning: the reference ships no golden vectors for this path (its
// example/regression tree is not part of the repository).  The oracle is
// pinned by the reference's own in-code known answers instead:
//   * the Gauss-Legendre self-check, basis_routines.f90:5886-5895
//   * the finite-difference element Jacobian rule,
//     equations_set_routines.f90:3032-3150 (delta=(1+||x||_2)*1e-7)
//   * closed-form homogeneous deformations (uniaxial stretch of the
//     incompressible MR law with sigma = dev(sigma_bar) + p I,
//     finite_elasticity_routines.f90:4386-4414)
// and by structural checks (symmetry, sparsity rule).
//
// Reference files followed (paths relative to the reference repository):
//   src/basis_routines.f90        GAUSS_LEGENDRE :5826-5903,
//                                 BASIS_QUADRATURE_CREATE :2770-2900,
//                                 BASIS_LHTP_BASIS_EVALUATE_DP :2251-2374,
//                                 LAGRANGE_LINEAR/QUADRATIC_EVALUATE :7015-7130,
//                                 BASIS_INTERPOLATE_GAUSS_DP :1123-1177
//   src/field_routines.f90        FIELD_INTERPOLATE_GAUSS :6071-6282
//   src/coordinate_routines.f90   COORDINATE_METRICS_CALCULATE :647-833,
//                                 Coordinates_MaterialSystemCalculate :3883-3981,
//                                 ..dXdNu3D :4042-4149
//   src/maths.f90                 INVERT_FULL_DP :1455-1521, CROSS_PRODUCT_DP
//                                 :333-367, MATRIX_PRODUCT_DP :1878-1921,
//                                 NORMALISE_DP :2059-2085, L2NORM_DP :1807-1821
//   src/constants.f90             ZERO_TOLERANCE :68, TENSOR_TO_VOIGT3 :284,
//                                 VOIGT_TO_TENSOR3 :285
//   src/finite_elasticity_routines.f90
//       FINITE_ELASTICITY_GAUSS_ELASTICITY_TENSOR   :609-835
//       FiniteElasticity_FiniteElementJacobianEvaluate :842-1175
//       FINITE_ELASTICITY_PUSH_ELASTICITY/STRESS_TENSOR :1182-1253
//       FiniteElasticity_FiniteElementResidualEvaluate :1260-1639
//       FiniteElasticity_GaussDeformationGradientTensor :3368-3425
//       FINITE_ELASTICITY_GAUSS_STRESS_TENSOR :4342-4454
//   src/equations_matrices_routines.f90
//       JacobianMatrix_StructureCalculate :5048-5340 (CSR sparsity rule)
//       EQUATIONS_MATRICES_JACOBIAN_ELEMENT_ADD :3174-3225
//   src/matrix_vector.f90         MATRIX_VALUES_ADD_DP2 CSR branch :2839-2876,
//                                 bisectionToLinearSearchThreshold :172
//   src/generated_mesh_routines.f90
//       GENERATED_MESH_REGULAR_CREATE_FINISH :1386-1600 (numbering),
//       GeneratedMesh_RegularComponentNodesToUserNumbers :5043-5200
//   src/mesh_routines.f90         MeshTopologyNodesCalculate :9006-9119
//                                 (mesh-component nodes in sorted order)
//   src/equations_set_routines.f90 FD Jacobian :3032-3150
// ============================================================================
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

extern "C" {

// Problem description consumed by the oracle.  Geometry, fibres and the
// displacement components share mesh component 1 (the u basis); a nodal
// pressure uses mesh component 2 (trilinear).
struct OrProblem {
  int32_t ne;               // number of elements
  int32_t nu;               // number of nodes of mesh component 1 (u)
  int32_t np;               // number of pressure nodes (0: element-constant p)
  int32_t nxi_u;            // nodes per xi direction of the u basis (2 or 3)
  int32_t p_mode;           // 0 element-based pressure, 1 nodal trilinear
  int32_t law;              // 1 Mooney-Rivlin, 15 Guccione (equations-set subtypes)
  int32_t nmat;             // materials components (2 MR, 4 Guccione)
  int32_t mat_per_element;  // 0 constant materials, 1 element-based materials
  const int32_t* elem_u;    // [ne][nxi_u^3] 0-based u node numbers
  const int32_t* elem_p;    // [ne][8] 0-based pressure node numbers (p_mode 1)
  const double* X;          // geometric field, [3][nu] component-major
  const double* mat;        // [nmat] or [ne][nmat]
  const double* fibre;      // nullable: fibre field angles [3][nu] (radians)
  const double* surf_p;     // nullable: surface pressure values [3][nu]; component n loads
                            // faces normal to xi_n (FIELD_PRESSURE_VALUES_SET_TYPE of DELUDELN)
  const uint8_t* bface;     // [ne][6] boundary-face flags (or_boundary_faces), needed with surf_p
};

}  // extern "C"

namespace {

const double ZERO_TOLERANCE = 5.0 * DBL_EPSILON;  // constants.f90:68
// TENSOR_TO_VOIGT3 (constants.f90:284), 0-based: 11->0 22->1 33->2 12->3 13->4 23->5
const int T2V[3][3] = {{0, 3, 4}, {3, 1, 5}, {4, 5, 2}};
// VOIGT_TO_TENSOR3 (constants.f90:285), 0-based pairs
const int V2T[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {0, 2}, {1, 2}};
const int NG = 27;  // 3x3x3 Gauss-Legendre

// ---------------------------------------------------------------- basis ----
// LAGRANGE_LINEAR_EVALUATE / LAGRANGE_QUADRATIC_EVALUATE, basis_routines.f90:7015-7130.
double lagrange(int order_nodes, int node /*1-based*/, int deriv, double xi) {
  if (order_nodes == 2) {
    if (deriv == 0) return node == 1 ? 1.0 - xi : xi;
    if (deriv == 1) return node == 1 ? -1.0 : 1.0;
    return 0.0;
  }
  if (deriv == 0) {
    if (node == 1) return 1.0 - 3.0 * xi + 2.0 * xi * xi;
    if (node == 2) return 4.0 * xi * (1.0 - xi);
    return xi * (xi + xi - 1.0);
  }
  if (deriv == 1) {
    if (node == 1) return 4.0 * xi - 3.0;
    if (node == 2) return 4.0 - 8.0 * xi;
    return 4.0 * xi - 1.0;
  }
  if (node == 2) return -8.0;
  return 4.0;
}

// Quadrature tables of one tensor-product Lagrange basis on the 3x3x3 Gauss
// scheme: GAUSS_BASIS_FNS(ns, nu, ng) with nu in {value, d/dxi1, d/dxi2,
// d/dxi3} (NO_PART_DERIV, PART_DERIV_S1/S2/S3 = 1,2,4,7 in the reference).
struct Tab {
  int n1 = 0, nn = 0;
  double gbf[NG][4][27];
  double w[NG];
  double xi[NG][3];
};

// GAUSS_LEGENDRE, basis_routines.f90:5826-5903, for 3 points on [0,1].
void gauss_legendre3(double x[3], double w[3]) {
  x[0] = (-std::sqrt(0.6) + 1.0) / 2.0;
  x[1] = 0.5;
  x[2] = (+std::sqrt(0.6) + 1.0) / 2.0;
  w[0] = 2.5 / 9.0;
  w[1] = 4.0 / 9.0;
  w[2] = 2.5 / 9.0;
}

// BASIS_QUADRATURE_CREATE (basis_routines.f90:2770-2900) with
// BASIS_LHTP_BASIS_EVALUATE_DP (:2251-2374): the product over xi directions
// is accumulated left to right starting from 1.0.
void build_tab(Tab& t, int n1) {
  t.n1 = n1;
  t.nn = n1 * n1 * n1;
  double gx[3], gw[3];
  gauss_legendre3(gx, gw);
  static const int dord[4][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  for (int k = 0; k < 3; ++k)
    for (int j = 0; j < 3; ++j)
      for (int i = 0; i < 3; ++i) {
        int ng = i + (j + k * 3) * 3;
        t.w[ng] = gw[i] * gw[j] * gw[k];
        double xi[3] = {gx[i], gx[j], gx[k]};
        for (int c = 0; c < 3; ++c) t.xi[ng][c] = xi[c];
        for (int nn = 0; nn < t.nn; ++nn) {
          int pos[3] = {nn % n1, (nn / n1) % n1, nn / (n1 * n1)};
          for (int nu = 0; nu < 4; ++nu) {
            double v = 1.0;
            for (int ni = 0; ni < 3; ++ni) v = v * lagrange(n1, pos[ni] + 1, dord[nu][ni], xi[ni]);
            t.gbf[ng][nu][nn] = v;
          }
        }
      }
}

const Tab& tab(int n1) {
  static Tab t2, t3;
  static bool init = false;
  if (!init) {
    build_tab(t2, 2);
    build_tab(t3, 3);
    init = true;
  }
  return n1 == 2 ? t2 : t3;
}

// ---------------------------------------------------------------- maths ----
// INVERT_FULL_DP 3x3 branch, maths.f90:1484-1498.  a is A(row,col).
void invert3(const double A[3][3], double B[3][3], double* det_out) {
  double det = A[0][0] * A[1][1] * A[2][2] + A[0][1] * A[1][2] * A[2][0] + A[0][2] * A[1][0] * A[2][1] -
               A[0][0] * A[2][1] * A[1][2] - A[1][0] * A[0][1] * A[2][2] - A[2][0] * A[1][1] * A[0][2];
  *det_out = det;
  if (std::fabs(det) > ZERO_TOLERANCE) {
    B[0][0] = (A[1][1] * A[2][2] - A[2][1] * A[1][2]) / det;
    B[1][0] = (A[1][2] * A[2][0] - A[2][2] * A[1][0]) / det;
    B[2][0] = (A[1][0] * A[2][1] - A[2][0] * A[1][1]) / det;
    B[0][1] = (A[2][1] * A[0][2] - A[0][1] * A[2][2]) / det;
    B[1][1] = (A[2][2] * A[0][0] - A[0][2] * A[2][0]) / det;
    B[2][1] = (A[2][0] * A[0][1] - A[0][0] * A[2][1]) / det;
    B[0][2] = (A[0][1] * A[1][2] - A[1][1] * A[0][2]) / det;
    B[1][2] = (A[0][2] * A[1][0] - A[1][2] * A[0][0]) / det;
    B[2][2] = (A[0][0] * A[1][1] - A[1][0] * A[0][1]) / det;
  } else {
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) B[i][j] = 0.0;
  }
}

// MATRIX_PRODUCT_DP 3x3 branch, maths.f90:1878-1921.
void matprod3(const double A[3][3], const double B[3][3], double C[3][3]) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) C[i][j] = A[i][0] * B[0][j] + A[i][1] * B[1][j] + A[i][2] * B[2][j];
}

// CROSS_PRODUCT_DP, maths.f90:333-367.
void cross3(const double a[3], const double b[3], double c[3]) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}

// NORMALISE_DP with L2NORM_DP, maths.f90:2059-2085, :1807-1821.
bool normalise3(const double a[3], double out[3]) {
  double s = 0.0;
  for (int i = 0; i < 3; ++i) s = s + a[i] * a[i];
  double len = std::sqrt(s);
  if (std::fabs(len) < ZERO_TOLERANCE) {
    for (int i = 0; i < 3; ++i) out[i] = a[i];
    return false;
  }
  for (int i = 0; i < 3; ++i) out[i] = a[i] / len;
  return true;
}

// ------------------------------------------------------- per-GP kinematics --
struct Metrics {
  double dxdxi[3][3];  // DX_DXI(coord, xi)
  double dxidx[3][3];  // DXI_DX(xi, coord)
  double jac;          // sqrt|det GL| (COORDINATE_JACOBIAN_VOLUME_TYPE)
};

// COORDINATE_METRICS_CALCULATE, rectangular cartesian 3-D, coordinate_routines.f90:647-833.
void metrics(Metrics& m) {
  double GL[3][3], GU[3][3], det_gl, det_dxdxi;
  for (int mi = 0; mi < 3; ++mi)
    for (int ni = 0; ni < 3; ++ni)
      GL[mi][ni] = m.dxdxi[0][mi] * m.dxdxi[0][ni] + m.dxdxi[1][mi] * m.dxdxi[1][ni] + m.dxdxi[2][mi] * m.dxdxi[2][ni];
  invert3(GL, GU, &det_gl);
  m.jac = std::sqrt(std::fabs(det_gl));
  invert3(m.dxdxi, m.dxidx, &det_dxdxi);
}

// Coordinates_MaterialSystemCalculatedXdNu3D, coordinate_routines.f90:4042-4149.
void dxdnu3d(const double dxdxi[3][3], const double ang[3], double dXdNu[3][3]) {
  double f[3], g[3], h[3], c1[3], c2[3];
  for (int i = 0; i < 3; ++i) {
    f[i] = dxdxi[i][0];
    c1[i] = dxdxi[i][0];
    c2[i] = dxdxi[i][1];
  }
  cross3(c1, c2, h);
  cross3(h, f, g);
  double R[3][3], nf[3], ng[3], nh[3];
  normalise3(f, nf);
  normalise3(g, ng);
  normalise3(h, nh);
  for (int i = 0; i < 3; ++i) {
    R[i][0] = nf[i];
    R[i][1] = ng[i];
    R[i][2] = nh[i];
  }
  double Rb[3][3], T3[3][3], T2[3][3];
  auto ident = [](double M[3][3]) {
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) M[i][j] = (i == j) ? 1.0 : 0.0;
  };
  ident(Rb);
  Rb[0][0] = std::cos(ang[0]);
  Rb[0][1] = -1.0 * std::sin(ang[0]);
  Rb[1][0] = std::sin(ang[0]);
  Rb[1][1] = std::cos(ang[0]);
  matprod3(R, Rb, T3);
  ident(Rb);
  Rb[0][0] = std::cos(ang[1]);
  Rb[0][2] = std::sin(ang[1]);
  Rb[2][0] = -1.0 * std::sin(ang[1]);
  Rb[2][2] = std::cos(ang[1]);
  matprod3(T3, Rb, T2);
  ident(Rb);
  Rb[1][1] = std::cos(ang[2]);
  Rb[1][2] = -1.0 * std::sin(ang[2]);
  Rb[2][1] = std::sin(ang[2]);
  Rb[2][2] = std::cos(ang[2]);
  matprod3(T2, Rb, dXdNu);
}

// Coordinates_MaterialSystemCalculate (coordinate_routines.f90:3883-3981):
// dXi/dNu from the geometric metrics and (optionally) the fibre angles.
void material_system(const Metrics& geo, const double* ang, double dXidNu[3][3]) {
  double dNudXi[3][3], det;
  if (ang) {
    double dXdNu[3][3], dNudX[3][3];
    dxdnu3d(geo.dxdxi, ang, dXdNu);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) dNudX[i][j] = dXdNu[j][i];
    matprod3(dNudX, geo.dxdxi, dNudXi);
  } else {
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) dNudXi[i][j] = geo.dxdxi[i][j];
  }
  invert3(dNudXi, dXidNu, &det);
}

// FINITE_ELASTICITY_PUSH_STRESS/ELASTICITY_TENSOR transform t(F), :1182-1253.
void push_t(const double F[3][3], double t[6][6]) {
  for (int j = 0; j < 3; ++j)
    for (int i = 0; i < 6; ++i) t[i][j] = F[V2T[i][0]][V2T[j][0]] * F[V2T[i][1]][V2T[j][1]];
  for (int j = 3; j < 6; ++j)
    for (int i = 0; i < 6; ++i)
      t[i][j] = F[V2T[i][0]][V2T[j][0]] * F[V2T[i][1]][V2T[j][1]] + F[V2T[i][0]][V2T[j][1]] * F[V2T[i][1]][V2T[j][0]];
}

void push_stress(double S[6], const double F[3][3], double J) {
  double t[6][6], r[6];
  push_t(F, t);
  for (int i = 0; i < 6; ++i) {
    double s = 0.0;
    for (int j = 0; j < 6; ++j) s = s + t[i][j] * S[j];
    r[i] = s;
  }
  for (int i = 0; i < 6; ++i) S[i] = r[i] / J;
}

void push_elasticity(double C[6][6], const double F[3][3], double J) {
  double t[6][6], A[6][6];
  push_t(F, t);
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j) {
      double s = 0.0;
      for (int k = 0; k < 6; ++k) s = s + t[i][k] * C[k][j];
      A[i][j] = s;
    }
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j) {
      double s = 0.0;
      for (int k = 0; k < 6; ++k) s = s + A[i][k] * t[j][k];
      C[i][j] = s / J;
    }
}

// MOD_DZDNU = F*J^(-1/3) and AZL = MOD^T MOD (:4369-4372 and :640-643).
void modified(const double F[3][3], double J, double mod[3][3], double azl[3][3]) {
  double s = std::pow(J, -1.0 / 3.0);
  double modt[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) mod[i][j] = F[i][j] * s;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) modt[i][j] = mod[j][i];
  matprod3(modt, mod, azl);
}

// Fictitious 2nd Piola stress (Voigt) and, if C is non-null, the fictitious
// material elasticity tensor for MR (:4386-4394, :684-699) or Guccione
// (:4419-4424, :758-781).
void fictitious(int law, const double* c, const double azl[3][3], double S[6], double (*C)[6]) {
  if (law == 1) {
    double I1 = azl[0][0] + azl[1][1] + azl[2][2];
    double t1 = -2.0 * c[1];
    double t2 = 2.0 * (c[0] + I1 * c[1]);
    S[0] = t1 * azl[0][0] + t2;
    S[1] = t1 * azl[1][1] + t2;
    S[2] = t1 * azl[2][2] + t2;
    S[3] = t1 * azl[1][0];
    S[4] = t1 * azl[2][0];
    S[5] = t1 * azl[2][1];
    if (C) {
      for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) C[i][j] = 0.0;
      double a = 4.0 * c[1], b = -2.0 * c[1];
      C[1][0] = a; C[2][0] = a; C[0][1] = a; C[2][1] = a; C[0][2] = a; C[1][2] = a;
      C[3][3] = b; C[4][4] = b; C[5][5] = b;
    }
  } else {
    double B[6] = {2.0 * c[1], 2.0 * c[2], 2.0 * c[2], c[3], c[3], c[2]};
    double E[6] = {0.5 * (azl[0][0] - 1.0), 0.5 * (azl[1][1] - 1.0), 0.5 * (azl[2][2] - 1.0),
                   azl[1][0], azl[2][0], azl[2][1]};
    double DQ[6];
    for (int i = 0; i < 6; ++i) DQ[i] = B[i] * E[i];
    double dot = 0.0;
    for (int i = 0; i < 6; ++i) dot = dot + E[i] * DQ[i];
    double t1 = 0.5 * c[0] * std::exp(0.5 * dot);
    for (int i = 0; i < 6; ++i) S[i] = t1 * DQ[i];
    if (C) {
      for (int j = 0; j < 6; ++j)
        for (int i = j; i < 6; ++i) C[i][j] = t1 * DQ[i] * DQ[j];
      for (int i = 0; i < 6; ++i) C[i][i] = C[i][i] + t1 * B[i];
      for (int j = 1; j < 6; ++j)
        for (int i = 0; i < j; ++i) C[i][j] = C[j][i];
    }
  }
}

// FINITE_ELASTICITY_GAUSS_STRESS_TENSOR (:4342-4454): Cauchy stress, Voigt.
void gauss_stress(int law, const double* c, const double F[3][3], double J, double p, double S[6]) {
  double mod[3][3], azl[3][3];
  modified(F, J, mod, azl);
  fictitious(law, c, azl, S, nullptr);
  push_stress(S, mod, J);
  double ot = (S[0] + S[1] + S[2]) / 3.0;
  for (int i = 0; i < 3; ++i) S[i] = S[i] - ot + p;
}

// FINITE_ELASTICITY_GAUSS_ELASTICITY_TENSOR (:609-835): spatial tangent and
// Cauchy stress, Voigt.
void gauss_elasticity(int law, const double* c, const double F[3][3], double J, double p, double C[6][6],
                      double S[6]) {
  const double ONETHIRD = 1.0 / 3.0, TWOTHIRDS = 2.0 / 3.0;
  const double DP11[3][3] = {{TWOTHIRDS, -ONETHIRD, -ONETHIRD},
                             {-ONETHIRD, TWOTHIRDS, -ONETHIRD},
                             {-ONETHIRD, -ONETHIRD, TWOTHIRDS}};
  const double TT_UNITY[6] = {TWOTHIRDS, TWOTHIRDS, TWOTHIRDS, 0.0, 0.0, 0.0};
  const double UNITY_DIAG[6] = {1.0, 1.0, 1.0, 0.5, 0.5, 0.5};
  double mod[3][3], azl[3][3];
  modified(F, J, mod, azl);
  fictitious(law, c, azl, S, C);
  push_stress(S, mod, J);
  push_elasticity(C, mod, J);
  double trace = S[0] + S[1] + S[2];
  for (int i = 0; i < 3; ++i) S[i] = S[i] - ONETHIRD * trace;
  double tt = TWOTHIRDS * trace;
  for (int i = 0; i < 6; ++i) C[i][i] = C[i][i] + tt * UNITY_DIAG[i];
  double M[3][3], N[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 0.0;
      for (int k = 0; k < 3; ++k) s = s + C[i][k] * DP11[k][j];
      M[i][j] = s;
    }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 0.0;
      for (int k = 0; k < 3; ++k) s = s + DP11[i][k] * M[k][j];
      N[i][j] = s;
    }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) C[i][j] = N[i][j];
  double T[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 0.0;
      for (int k = 0; k < 3; ++k) s = s + DP11[i][k] * C[k][3 + j];
      T[i][j] = s;
    }
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      C[i][3 + j] = T[i][j];
      C[3 + j][i] = T[i][j];
    }
  for (int j = 0; j < 6; ++j)
    for (int i = 0; i < 6; ++i) C[i][j] = C[i][j] - (TT_UNITY[i] * S[j] + TT_UNITY[j] * S[i]);
  for (int i = 0; i < 3; ++i) S[i] = S[i] + p;
  for (int i = 0; i < 6; ++i) C[i][i] = C[i][i] - p;
  C[1][0] = C[1][0] + p; C[2][0] = C[2][0] + p; C[0][1] = C[0][1] + p;
  C[2][1] = C[2][1] + p; C[0][2] = C[0][2] + p; C[1][2] = C[1][2] + p;
}

// ---------------------------------------------------------- element data ----
struct Elem {
  int npe, npp;        // u parameters per component, pressure parameters
  int nrow;            // 3*npe + npp
  double z[27][3], X[27][3], fib[27][3], p[8];
  const double* c;
  const Tab* tu;
  const Tab* tp;
};

// FIELD_INTERPOLATION_PARAMETERS_ELEMENT_GET, no-scaling branch (field_routines.f90:8443-8455).
void gather(const OrProblem* P, int e, const double* x, Elem& E) {
  E.tu = &tab(P->nxi_u);
  E.tp = &tab(2);
  E.npe = E.tu->nn;
  E.npp = P->p_mode ? 8 : 1;
  E.nrow = 3 * E.npe + E.npp;
  const int nu = P->nu;
  for (int a = 0; a < E.npe; ++a) {
    int node = P->elem_u[(size_t)e * E.npe + a];
    for (int c = 0; c < 3; ++c) {
      E.z[a][c] = x[(size_t)c * nu + node];
      E.X[a][c] = P->X[(size_t)c * nu + node];
      E.fib[a][c] = P->fibre ? P->fibre[(size_t)c * nu + node] : 0.0;
    }
  }
  if (P->p_mode)
    for (int q = 0; q < 8; ++q) E.p[q] = x[(size_t)3 * nu + P->elem_p[(size_t)e * 8 + q]];
  else
    E.p[0] = x[(size_t)3 * nu + e];
  E.c = P->mat_per_element ? P->mat + (size_t)e * P->nmat : P->mat;
}

// BASIS_INTERPOLATE_GAUSS_DP (basis_routines.f90:1123-1177): sum over ns from 0.
double interp(const Tab& t, int g, int nu, const double* prm, int stride) {
  double s = 0.0;
  for (int ns = 0; ns < t.nn; ++ns) s = s + t.gbf[g][nu][ns] * prm[ns * stride];
  return s;
}

struct GP {
  Metrics dep, geo;
  double F[3][3];
  double p, Jznu;
};

void gp_kinematics(const OrProblem* P, const Elem& E, int g, GP& G) {
  const Tab& t = *E.tu;
  for (int c = 0; c < 3; ++c)
    for (int k = 0; k < 3; ++k) {
      G.dep.dxdxi[c][k] = interp(t, g, k + 1, &E.z[0][c], 3);
      G.geo.dxdxi[c][k] = interp(t, g, k + 1, &E.X[0][c], 3);
    }
  G.p = P->p_mode ? interp(*E.tp, g, 0, E.p, 1) : E.p[0];
  metrics(G.dep);
  metrics(G.geo);
  double ang[3];
  const double* angp = nullptr;
  if (P->fibre) {
    for (int c = 0; c < 3; ++c) ang[c] = interp(t, g, 0, &E.fib[0][c], 3);
    angp = ang;
  }
  double dXidNu[3][3];
  material_system(G.geo, angp, dXidNu);
  matprod3(G.dep.dxdxi, dXidNu, G.F);  // FiniteElasticity_GaussDeformationGradientTensor
  G.Jznu = G.dep.jac / G.geo.jac;
}

// Local faces in the reference's order (basis_routines.f90:2162-2224): the
// -xi faces for xi = 1,2,3, then the +xi faces.  Face nodes run along the
// first in-face direction fastest (OTHER_XI_DIRECTIONS3, constants.f90:270):
// normal xi1 -> (xi2, xi3), xi2 -> (xi1, xi3), xi3 -> (xi1, xi2).
void face_info(int lf, int n1, int& ni, int& side, int& xa, int& xb, int nodes[9]) {
  ni = lf % 3;
  side = lf / 3;
  xa = ni == 0 ? 1 : 0;
  xb = ni == 2 ? 1 : 2;
  for (int f2 = 0; f2 < n1; ++f2)
    for (int f1 = 0; f1 < n1; ++f1) {
      int pos[3];
      pos[ni] = side ? n1 - 1 : 0;
      pos[xa] = f1;
      pos[xb] = f2;
      nodes[f1 + n1 * f2] = pos[0] + n1 * (pos[1] + n1 * pos[2]);
    }
}

// Face quadrature tables: 3x3 Gauss-Legendre on the face, point ng = i + 3j.
struct FaceTab {
  double w[9], N[9][9], dN[9][2][9];
};
const FaceTab& face_tab(int n1) {
  static FaceTab t[2];
  static bool init = false;
  if (!init) {
    double gx[3], gw[3];
    gauss_legendre3(gx, gw);
    for (int k = 0; k < 2; ++k) {
      const int m = k + 2;
      for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i) {
          const int ng = i + 3 * j;
          t[k].w[ng] = gw[i] * gw[j];
          for (int f2 = 0; f2 < m; ++f2)
            for (int f1 = 0; f1 < m; ++f1) {
              const int f = f1 + m * f2;
              t[k].N[ng][f] = 1.0 * lagrange(m, f1 + 1, 0, gx[i]) * lagrange(m, f2 + 1, 0, gx[j]);
              t[k].dN[ng][0][f] = 1.0 * lagrange(m, f1 + 1, 1, gx[i]) * lagrange(m, f2 + 1, 0, gx[j]);
              t[k].dN[ng][1][f] = 1.0 * lagrange(m, f1 + 1, 0, gx[i]) * lagrange(m, f2 + 1, 1, gx[j]);
            }
        }
    }
    init = true;
  }
  return t[n1 - 2];
}

// FiniteElasticity_SurfacePressureResidualEvaluate (finite_elasticity_routines.f90:3215-3361) when re,
// FiniteElasticity_SurfacePressureJacobianEvaluate (:3049-3208) when Ke (column-major, lower
// off-diagonal displacement blocks only, before the element matrix is mirrored).
void surface_pressure(const OrProblem* P, int e, const Elem& E, double* re, double* Ke, int n) {
  if (!P->surf_p || !P->bface) return;
  const int n1 = P->nxi_u, nf = n1 * n1, npe = E.npe;
  const FaceTab& T = face_tab(n1);
  static const int ORIENT[3] = {1, -1, 1};  // OTHER_XI_ORIENTATIONS3 of the in-face pair
  for (int lf = 0; lf < 6; ++lf) {
    if (!P->bface[(size_t)e * 6 + lf]) continue;
    int ni, side, xa, xb, fn[9];
    face_info(lf, n1, ni, side, xa, xb, fn);
    double pf[9];
    bool nonzero = false;
    for (int f = 0; f < nf; ++f) {
      pf[f] = P->surf_p[(size_t)ni * P->nu + P->elem_u[(size_t)e * npe + fn[f]]];
      if (std::fabs(pf[f]) > ZERO_TOLERANCE) nonzero = true;
    }
    if (!nonzero) continue;
    const int orientation = (side ? 1 : -1) * ORIENT[ni] > 0 ? 1 : -1;
    for (int ng = 0; ng < 9; ++ng) {
      double p = 0.0, g[3][2];
      for (int f = 0; f < nf; ++f) p = p + T.N[ng][f] * pf[f];
      for (int c = 0; c < 3; ++c)
        for (int d = 0; d < 2; ++d) {
          double s = 0.0;
          for (int f = 0; f < nf; ++f) s = s + T.dN[ng][d][f] * E.z[fn[f]][c];
          g[c][d] = s;
        }
      // COORDINATE_METRICS_CALCULATE, surface in 3-D space (coordinate_routines.f90:908-915)
      double GL[2][2];
      for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b) GL[a][b] = g[0][a] * g[0][b] + g[1][a] * g[1][b] + g[2][a] * g[2][b];
      const double det_gl = GL[0][0] * GL[1][1] - GL[1][0] * GL[0][1];
      double dxi[2][3];
      for (int c = 0; c < 3; ++c) {
        dxi[0][c] = (GL[1][1] * g[c][0] - GL[0][1] * g[c][1]) / det_gl;
        dxi[1][c] = (GL[0][0] * g[c][1] - GL[1][0] * g[c][0]) / det_gl;
      }
      double a1[3] = {g[0][0], g[1][0], g[2][0]}, a2[3] = {g[0][1], g[1][1], g[2][1]}, nrm[3];
      cross3(a1, a2, nrm);
      const double pg = p * orientation;
      const double gwp = T.w[ng] * pg;
      if (re) {
        for (int c = 0; c < 3; ++c) {
          const double gpn = gwp * nrm[c];
          for (int f = 0; f < nf; ++f) re[c * npe + fn[f]] = re[c * npe + fn[f]] + gpn * T.N[ng][f];
        }
      }
      if (Ke) {
        static const int OD[3][2] = {{0, 1}, {0, 2}, {1, 2}};
        for (int oh = 0; oh < 3; ++oh) {
          const int nh = OD[oh][0], mh = OD[oh][1];
          double W[2];
          for (int i = 0; i < 2; ++i) W[i] = (nrm[mh] * dxi[i][nh] - dxi[i][mh] * nrm[nh]) * gwp;
          for (int ns = 0; ns < nf; ++ns) {
            const double t1[2] = {W[0] * T.dN[ng][0][ns], W[1] * T.dN[ng][1][ns]};
            const int col = nh * npe + fn[ns];
            for (int ms = 0; ms < nf; ++ms) {
              const double t2 = T.N[ng][ms];
              const int row = mh * npe + fn[ms];
              Ke[(size_t)col * n + row] = Ke[(size_t)col * n + row] + (t1[0] * t2 + t1[1] * t2);
            }
          }
        }
      }
    }
  }
}

}  // namespace

extern "C" {

// Boundary faces: a local face whose corner nodes no other element holds
// (DECOMPOSITION face BOUNDARY_FACE).  flags has [ne][6] entries.
void or_boundary_faces(const OrProblem* P, uint8_t* flags) {
  const int n1 = P->nxi_u, npe = n1 * n1 * n1;
  std::vector<std::vector<int>> surr(P->nu);
  for (int e = 0; e < P->ne; ++e)
    for (int a = 0; a < npe; ++a) surr[P->elem_u[(size_t)e * npe + a]].push_back(e);
  for (int e = 0; e < P->ne; ++e)
    for (int lf = 0; lf < 6; ++lf) {
      int ni, side, xa, xb, fn[9];
      face_info(lf, n1, ni, side, xa, xb, fn);
      const int nf = n1 * n1;
      int corners[4] = {P->elem_u[(size_t)e * npe + fn[0]], P->elem_u[(size_t)e * npe + fn[n1 - 1]],
                        P->elem_u[(size_t)e * npe + fn[nf - n1]], P->elem_u[(size_t)e * npe + fn[nf - 1]]};
      bool shared = false;
      for (int f : surr[corners[0]]) {
        if (f == e) continue;
        int hit = 0;
        for (int k = 0; k < 4; ++k)
          for (int a = 0; a < npe; ++a)
            if (P->elem_u[(size_t)f * npe + a] == corners[k]) {
              ++hit;
              break;
            }
        if (hit == 4) shared = true;
      }
      flags[(size_t)e * 6 + lf] = shared ? 0 : 1;
    }
}

// Number of element rows (3*npe_u + npe_p).
int or_element_size(const OrProblem* P) {
  int npe = P->nxi_u * P->nxi_u * P->nxi_u;
  return 3 * npe + (P->p_mode ? 8 : 1);
}

// FiniteElasticity_FiniteElementResidualEvaluate, MR/Guccione branch
// (finite_elasticity_routines.f90:1488-1604).  re has or_element_size() entries.
void or_element_residual(const OrProblem* P, int e, const double* x, double* re) {
  Elem E;
  gather(P, e, x, E);
  for (int i = 0; i < E.nrow; ++i) re[i] = 0.0;
  const Tab& t = *E.tu;
  double dphidz[3][27][3];  // DPHIDZ(mh, ns, nh) stored as [nh][ns][mh]
  for (int g = 0; g < NG; ++g) {
    GP G;
    gp_kinematics(P, E, g, G);
    for (int nh = 0; nh < 3; ++nh)
      for (int ns = 0; ns < E.npe; ++ns)
        for (int mh = 0; mh < 3; ++mh) {
          double s = 0.0;
          for (int mi = 0; mi < 3; ++mi) s = s + G.dep.dxidx[mi][mh] * t.gbf[g][mi + 1][ns];
          dphidz[nh][ns][mh] = s;
        }
    double jgw = G.dep.jac * t.w[g];
    double S[6];
    gauss_stress(P->law, E.c, G.F, G.Jznu, G.p, S);
    double jc[3][3];
    for (int nh = 0; nh < 3; ++nh)
      for (int mh = 0; mh < 3; ++mh) jc[mh][nh] = jgw * S[T2V[mh][nh]];
    int mhs = 0;
    for (int mh = 0; mh < 3; ++mh)
      for (int ms = 0; ms < E.npe; ++ms) {
        double d = 0.0;
        for (int i = 0; i < 3; ++i) d = d + dphidz[mh][ms][i] * jc[i][mh];
        re[mhs] = re[mhs] + d;
        ++mhs;
      }
    jgw = G.geo.jac * t.w[g];
    double t1 = jgw * (G.Jznu - 1.0);
    if (P->p_mode) {
      for (int ms = 0; ms < 8; ++ms) {
        re[mhs] = re[mhs] + t1 * E.tp->gbf[g][0][ms];
        ++mhs;
      }
    } else {
      re[mhs] = re[mhs] + t1;
    }
  }
  surface_pressure(P, e, E, re, nullptr, E.nrow);
}

// FiniteElasticity_FiniteElementJacobianEvaluate (finite_elasticity_routines.f90:842-1175),
// without surface pressure or scale factors (no-scaling Lagrange fields).
// Ke is column-major [nrow x nrow] like ELEMENT_JACOBIAN%MATRIX(mhs,nhs).
void or_element_jacobian(const OrProblem* P, int e, const double* x, double* Ke) {
  Elem E;
  gather(P, e, x, E);
  const int n = E.nrow;
  for (int i = 0; i < n * n; ++i) Ke[i] = 0.0;
  auto K = [&](int r, int c) -> double& { return Ke[(size_t)c * n + r]; };
  const Tab& t = *E.tu;
  const int npe = E.npe;
  const int base[4] = {0, npe, 2 * npe, 3 * npe};
  double dphidz[3][27][3];
  for (int g = 0; g < NG; ++g) {
    GP G;
    gp_kinematics(P, E, g, G);
    double jgw = G.dep.jac * t.w[g];
    for (int nh = 0; nh < 3; ++nh)
      for (int ns = 0; ns < npe; ++ns)
        for (int mh = 0; mh < 3; ++mh) {
          double s = 0.0;
          for (int ni = 0; ni < 3; ++ni) s = s + t.gbf[g][ni + 1][ns] * G.dep.dxidx[ni][mh];
          dphidz[nh][ns][mh] = s;
        }
    double C[6][6], S[6];
    gauss_elasticity(P->law, E.c, G.F, G.Jznu, G.p, C, S);
    double cauchy[3][3];
    for (int nh = 0; nh < 3; ++nh)
      for (int mh = 0; mh < 3; ++mh) cauchy[mh][nh] = S[T2V[mh][nh]];
    // 1) mh == nh blocks, lower triangle
    for (int nh = 0; nh < 3; ++nh) {
      double sub[3][3];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) sub[i][j] = jgw * (C[T2V[i][nh]][T2V[j][nh]] + cauchy[i][j]);
      for (int ns = 0; ns < npe; ++ns) {
        double tv[3];
        for (int i = 0; i < 3; ++i) {
          double s = 0.0;
          for (int j = 0; j < 3; ++j) s = s + sub[i][j] * dphidz[nh][ns][j];
          tv[i] = s;
        }
        int col = base[nh] + ns;
        for (int ms = ns; ms < npe; ++ms) {
          double d = 0.0;
          for (int i = 0; i < 3; ++i) d = d + dphidz[nh][ms][i] * tv[i];
          K(base[nh] + ms, col) += d;
        }
      }
    }
    // 2) mh > nh blocks
    static const int OD[3][2] = {{0, 1}, {0, 2}, {1, 2}};
    for (int oh = 0; oh < 3; ++oh) {
      int nh = OD[oh][0], mh = OD[oh][1];
      double sub[3][3];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) sub[i][j] = jgw * C[T2V[i][mh]][T2V[j][nh]];
      for (int ns = 0; ns < npe; ++ns) {
        double tv[3];
        for (int i = 0; i < 3; ++i) {
          double s = 0.0;
          for (int j = 0; j < 3; ++j) s = s + sub[i][j] * dphidz[nh][ns][j];
          tv[i] = s;
        }
        int col = base[nh] + ns;
        for (int ms = 0; ms < npe; ++ms) {
          double d = 0.0;
          for (int i = 0; i < 3; ++i) d = d + dphidz[mh][ms][i] * tv[i];
          K(base[mh] + ms, col) += d;
        }
      }
    }
    // 3) pressure rows x displacement columns
    for (int nh = 0; nh < 3; ++nh)
      for (int ns = 0; ns < npe; ++ns) {
        double jd = jgw * dphidz[nh][ns][nh];
        int col = base[nh] + ns;
        if (P->p_mode) {
          for (int ms = 0; ms < 8; ++ms) K(base[3] + ms, col) += jd * E.tp->gbf[g][0][ms];
        } else {
          K(base[3], col) += jd;
        }
      }
  }
  // surface pressure follower load before the mirror (:1075-1078)
  surface_pressure(P, e, E, nullptr, Ke, n);
  // mirror the lower triangle (:1149-1153)
  for (int c = 1; c < n; ++c)
    for (int r = 0; r < c; ++r) K(r, c) = K(c, r);
}

// Element DOF numbers (0-based global), component-major like ELEMENT_MATRIX_CALCULATE
// (equations_matrices_routines.f90:684-940) for a single rank (local == global).
void or_element_dofs(const OrProblem* P, int e, int32_t* dofs) {
  int npe = P->nxi_u * P->nxi_u * P->nxi_u, k = 0;
  for (int c = 0; c < 3; ++c)
    for (int a = 0; a < npe; ++a) dofs[k++] = c * P->nu + P->elem_u[(size_t)e * npe + a];
  if (P->p_mode)
    for (int q = 0; q < 8; ++q) dofs[k++] = 3 * P->nu + P->elem_p[(size_t)e * 8 + q];
  else
    dofs[k++] = 3 * P->nu + e;
}

int64_t or_num_dofs(const OrProblem* P) { return (int64_t)3 * P->nu + (P->p_mode ? P->np : P->ne); }

// One-sided finite-difference element Jacobian with the reference's step rule
// (equations_set_routines.f90:3086-3130): delta=(1+||x||_2)*1e-7, one column
// per element parameter, using the element residual above.  x is modified and
// restored.
void or_element_jacobian_fd(const OrProblem* P, int e, double* x, double* Ke) {
  int n = or_element_size(P);
  int64_t nd = or_num_dofs(P);
  double s = 0.0;
  for (int64_t i = 0; i < nd; ++i) s += x[i] * x[i];
  double delta = (1.0 + std::sqrt(s)) * 1e-7;
  std::vector<double> r0(n), r1(n);
  std::vector<int32_t> dofs(n);
  or_element_dofs(P, e, dofs.data());
  or_element_residual(P, e, x, r0.data());
  for (int col = 0; col < n; ++col) {
    double orig = x[dofs[col]];
    x[dofs[col]] = orig + delta;
    or_element_residual(P, e, x, r1.data());
    x[dofs[col]] = orig;
    for (int r = 0; r < n; ++r) Ke[(size_t)col * n + r] = (r1[r] - r0[r]) / delta;
  }
}

// ------------------------------------------------------------- sparsity ----
// JacobianMatrix_StructureCalculate, compressed-row FEM branch
// (equations_matrices_routines.f90:5085-5300): for every row dof, the column
// list is the union of all dofs of all components of every element
// surrounding the row's node (or of the row's own element for an
// element-based component, plus its own diagonal), de-duplicated and sorted
// (LIST_REMOVE_DUPLICATES).  Output is 1-based (ROW_INDICES, COLUMN_INDICES).
// Two-call protocol: pass col == nullptr to receive only row_ptr and nnz.
int64_t or_pattern(const OrProblem* P, int32_t* row_ptr, int32_t* col) {
  const int npe = P->nxi_u * P->nxi_u * P->nxi_u;
  const int64_t nd = or_num_dofs(P);
  // surrounding elements of every node of each mesh component
  std::vector<std::vector<int>> surr_u(P->nu), surr_p(P->p_mode ? P->np : 0);
  for (int e = 0; e < P->ne; ++e) {
    for (int a = 0; a < npe; ++a) {
      auto& v = surr_u[P->elem_u[(size_t)e * npe + a]];
      if (v.empty() || v.back() != e) v.push_back(e);
    }
    if (P->p_mode)
      for (int q = 0; q < 8; ++q) {
        auto& v = surr_p[P->elem_p[(size_t)e * 8 + q]];
        if (v.empty() || v.back() != e) v.push_back(e);
      }
  }
  std::vector<int32_t> dofs(3 * npe + 8), list;
  int64_t nnz = 0;
  if (row_ptr) row_ptr[0] = 1;
  for (int64_t r = 0; r < nd; ++r) {
    list.clear();
    const std::vector<int>* elems;
    std::vector<int> own;
    bool elem_row = false;
    if (r < 3 * (int64_t)P->nu) {
      elems = &surr_u[r % P->nu];
    } else if (P->p_mode) {
      elems = &surr_p[r - 3 * (int64_t)P->nu];
    } else {
      own.push_back((int)(r - 3 * (int64_t)P->nu));
      elems = &own;
      elem_row = true;
    }
    for (int e : *elems) {
      or_element_dofs(P, e, dofs.data());
      int nrow = or_element_size(P);
      for (int k = 0; k < nrow; ++k) list.push_back(dofs[k]);
    }
    (void)elem_row;
    std::sort(list.begin(), list.end());
    list.erase(std::unique(list.begin(), list.end()), list.end());
    if (col)
      for (size_t k = 0; k < list.size(); ++k) col[nnz + k] = list[k] + 1;
    nnz += (int64_t)list.size();
    if (row_ptr) row_ptr[r + 1] = (int32_t)(nnz + 1);
  }
  return nnz;
}

// ------------------------------------------------------------- assembly ----
// MATRIX_VALUES_ADD_DP2, compressed-row branch (matrix_vector.f90:2839-2876):
// per element row, bisection down to bisectionToLinearSearchThreshold=10
// entries, then a linear scan; 1-based CSR.  Returns 0, or -1 if a slot is
// missing (the reference raises "does not exist in the matrix").
static int csr_add_element(const int32_t* rp, const int32_t* ci, int64_t nnz, double* val, const int32_t* rows,
                           const int32_t* cols, int n, const double* Ke) {
  const int THRESH = 10;
  int64_t prev = -1;
  for (int i = 0; i < n; ++i) {
    int64_t row = rows[i] + 1;  // 1-based
    int64_t lo = rp[row - 1], up = rp[row];
    for (int j = 0; j < n; ++j) {
      int64_t loc = 0, cidx = cols[j] + 1;
      if (cidx <= prev)
        lo = rp[row - 1];
      else
        up = rp[row];
      prev = cidx;
      while (up - lo > THRESH) {
        int64_t mid = (up + lo) / 2;
        if (ci[mid - 1] > cidx)
          up = mid;
        else
          lo = mid;
      }
      for (int64_t k = lo; k <= up && k <= nnz; ++k)
        if (ci[k - 1] == cidx) {
          loc = k;
          lo = k + 1;
          break;
        }
      if (loc == 0) return -1;
      val[loc - 1] = val[loc - 1] + Ke[(size_t)j * n + i];
    }
  }
  return 0;
}

// Greedy element colouring: no two elements of a colour share a node of any
// mesh component.  Used only by the multi-threaded CPU baseline below.
static int colour_elements(const OrProblem* P, std::vector<int>& colour) {
  const int npe = P->nxi_u * P->nxi_u * P->nxi_u;
  std::vector<uint64_t> umask(P->nu, 0), pmask(P->p_mode ? P->np : 0, 0);
  colour.assign(P->ne, 0);
  int ncol = 0;
  for (int e = 0; e < P->ne; ++e) {
    uint64_t used = 0;
    for (int a = 0; a < npe; ++a) used |= umask[P->elem_u[(size_t)e * npe + a]];
    if (P->p_mode)
      for (int q = 0; q < 8; ++q) used |= pmask[P->elem_p[(size_t)e * 8 + q]];
    int c = 0;
    while (c < 63 && (used >> c & 1)) ++c;
    colour[e] = c;
    ncol = std::max(ncol, c + 1);
    for (int a = 0; a < npe; ++a) umask[P->elem_u[(size_t)e * npe + a]] |= (1ull << c);
    if (P->p_mode)
      for (int q = 0; q < 8; ++q) pmask[P->elem_p[(size_t)e * 8 + q]] |= (1ull << c);
  }
  return ncol;
}

// EQUATIONS_SET_{JACOBIAN,RESIDUAL}_EVALUATE_STATIC_FEM (equations_set_routines.f90:4878-5024,
// :5483-5640): zero the Jacobian values and the residual, then for every
// element evaluate the element Jacobian/residual and add them into the CSR
// matrix (bisection add) and the residual vector.  nthreads == 1 follows the
// reference's serial element order; nthreads > 1 processes element colours in
// sequence with the elements of one colour split across threads.
// values (nnz) and/or residual (ndofs) may be null to skip that part.
int or_assemble(const OrProblem* P, const double* x, const int32_t* rp, const int32_t* ci, double* values,
                double* residual, int nthreads) {
  const int n = or_element_size(P);
  const int64_t nd = or_num_dofs(P);
  const int64_t nnz = rp[nd] - 1;
  if (values)
    for (int64_t k = 0; k < nnz; ++k) values[k] = 0.0;
  if (residual)
    for (int64_t k = 0; k < nd; ++k) residual[k] = 0.0;
  auto do_elem = [&](int e, std::vector<double>& Ke, std::vector<double>& re, std::vector<int32_t>& dofs) -> int {
    or_element_dofs(P, e, dofs.data());
    if (values) {
      or_element_jacobian(P, e, x, Ke.data());
      if (csr_add_element(rp, ci, nnz, values, dofs.data(), dofs.data(), n, Ke.data())) return -1;
    }
    if (residual) {
      or_element_residual(P, e, x, re.data());
      for (int i = 0; i < n; ++i) residual[dofs[i]] = residual[dofs[i]] + re[i];
    }
    return 0;
  };
  if (nthreads <= 1) {
    std::vector<double> Ke((size_t)n * n), re(n);
    std::vector<int32_t> dofs(n);
    for (int e = 0; e < P->ne; ++e)
      if (do_elem(e, Ke, re, dofs)) return -1;
    return 0;
  }
  std::vector<int> colour;
  int ncol = colour_elements(P, colour);
  std::vector<std::vector<int>> lists(ncol);
  for (int e = 0; e < P->ne; ++e) lists[colour[e]].push_back(e);
  int err = 0;
  for (int c = 0; c < ncol; ++c) {
    const std::vector<int>& L = lists[c];
    std::vector<std::thread> th;
    std::vector<int> errs(nthreads, 0);
    for (int t = 0; t < nthreads; ++t)
      th.emplace_back([&, t]() {
        std::vector<double> Ke((size_t)n * n), re(n);
        std::vector<int32_t> dofs(n);
        for (size_t i = t; i < L.size(); i += nthreads)
          if (do_elem(L[i], Ke, re, dofs)) errs[t] = -1;
      });
    for (auto& h : th) h.join();
    for (int t = 0; t < nthreads; ++t) err |= errs[t];
  }
  return err ? -1 : 0;
}

// Timing sample of or_assemble: the elements first .. first+count-1 only,
// added into values / residual (not zeroed here), element colours in order,
// each colour's elements split over nthreads threads.
int or_assemble_range(const OrProblem* P, const double* x, const int32_t* rp, const int32_t* ci, double* values,
                      double* residual, int first, int count, int nthreads) {
  const int n = or_element_size(P);
  const int64_t nd = or_num_dofs(P);
  const int64_t nnz = rp[nd] - 1;
  if (first < 0 || count < 0 || first + count > P->ne) return -2;
  std::vector<int> colour;
  const int ncol = colour_elements(P, colour);
  std::vector<std::vector<int>> lists(ncol);
  for (int e = first; e < first + count; ++e) lists[colour[e]].push_back(e);
  if (nthreads < 1) nthreads = 1;
  int err = 0;
  for (int c = 0; c < ncol; ++c) {
    const std::vector<int>& L = lists[c];
    std::vector<std::thread> th;
    std::vector<int> errs(nthreads, 0);
    for (int t = 0; t < nthreads; ++t)
      th.emplace_back([&, t]() {
        std::vector<double> Ke((size_t)n * n), re(n);
        std::vector<int32_t> dofs(n);
        for (size_t i = t; i < L.size(); i += nthreads) {
          const int e = L[i];
          or_element_dofs(P, e, dofs.data());
          if (values) {
            or_element_jacobian(P, e, x, Ke.data());
            if (csr_add_element(rp, ci, nnz, values, dofs.data(), dofs.data(), n, Ke.data())) errs[t] = -1;
          }
          if (residual) {
            or_element_residual(P, e, x, re.data());
            for (int k = 0; k < n; ++k) residual[dofs[k]] = residual[dofs[k]] + re[k];
          }
        }
      });
    for (auto& h : th) h.join();
    for (int t = 0; t < nthreads; ++t) err |= errs[t];
  }
  return err ? -1 : 0;
}

// ------------------------------------------------------- regular meshes ----
// GENERATED_MESH_REGULAR_CREATE_FINISH for Lagrange tensor-product bases
// (generated_mesh_routines.f90:1480-1600): element numbering x fastest, element
// nodes x fastest, node numbers np + (nn1-1) + (nn2-1)*N1 + (nn3-1)*N1*N2.
// A second (trilinear) pressure basis takes its node user numbers from the
// corner nodes of the first basis (GeneratedMesh_RegularComponentNodesToUserNumbers,
// :5043-5200), and its mesh-component nodes are the sorted set of those user
// numbers (MeshTopologyNodesCalculate, mesh_routines.f90:9006-9119).
// Writes elem_u [ne][n1^3] and, if elem_p != null, elem_p [ne][8]; returns
// the number of pressure nodes (0 when elem_p is null).
int or_regular_mesh(int ex, int ey, int ez, int n1, int32_t* elem_u, int32_t* elem_p) {
  const int TN1 = (n1 - 1) * ex + 1, TN2 = (n1 - 1) * ey + 1;
  const int E[3] = {ex, ey, ez};
  const int npe = n1 * n1 * n1;
  for (int ne3 = 1; ne3 <= E[2] + 1; ++ne3)
    for (int ne2 = 1; ne2 <= E[1] + 1; ++ne2)
      for (int ne1 = 1; ne1 <= E[0] + 1; ++ne1) {
        if (!(ne3 <= E[2] && ne2 <= E[1] && ne1 <= E[0])) continue;
        int grid_ne = ne1 + (ne2 - 1) * E[0] + (ne3 - 1) * E[0] * E[1];
        int np = 1 + (ne1 - 1) * (n1 - 1) + (ne2 - 1) * TN1 * (n1 - 1) + (ne3 - 1) * TN1 * TN2 * (n1 - 1);
        int nn = 0;
        for (int nn3 = 1; nn3 <= n1; ++nn3)
          for (int nn2 = 1; nn2 <= n1; ++nn2)
            for (int nn1 = 1; nn1 <= n1; ++nn1) {
              elem_u[(size_t)(grid_ne - 1) * npe + nn] = np + (nn1 - 1) + (nn2 - 1) * TN1 + (nn3 - 1) * TN1 * TN2 - 1;
              ++nn;
            }
      }
  if (!elem_p) return 0;
  const int ne = ex * ey * ez;
  std::vector<int32_t> users((size_t)ne * 8);
  for (int e = 0; e < ne; ++e) {
    int k = 0;
    for (int nn3 = 0; nn3 < 2; ++nn3)
      for (int nn2 = 0; nn2 < 2; ++nn2)
        for (int nn1 = 0; nn1 < 2; ++nn1) {
          int first = (nn1 ? n1 - 1 : 0) + (nn2 ? (n1 - 1) * n1 : 0) + (nn3 ? n1 * n1 * (n1 - 1) : 0);
          users[(size_t)e * 8 + k++] = elem_u[(size_t)e * npe + first];
        }
  }
  std::vector<int32_t> sorted(users);
  std::sort(sorted.begin(), sorted.end());
  sorted.erase(std::unique(sorted.begin(), sorted.end()), sorted.end());
  for (size_t i = 0; i < users.size(); ++i)
    elem_p[i] = (int32_t)(std::lower_bound(sorted.begin(), sorted.end(), users[i]) - sorted.begin());
  return (int)sorted.size();
}

// Quadrature tables for tests: gbf [27][4][n1^3], weights [27], points [27][3].
void or_basis_tables(int n1, double* gbf, double* w, double* xi) {
  const Tab& t = tab(n1);
  for (int g = 0; g < NG; ++g) {
    if (w) w[g] = t.w[g];
    if (xi)
      for (int c = 0; c < 3; ++c) xi[g * 3 + c] = t.xi[g][c];
    if (gbf)
      for (int nu = 0; nu < 4; ++nu)
        for (int a = 0; a < t.nn; ++a) gbf[((size_t)g * 4 + nu) * t.nn + a] = t.gbf[g][nu][a];
  }
}

// Cauchy stress (Voigt) and spatial elasticity tensor at one point, for the
// closed-form patch tests.  F is row-major, J is det F.
void or_point_stress(int law, const double* c, const double* F, double J, double p, double* S, double* C) {
  double Fm[3][3];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) Fm[i][j] = F[i * 3 + j];
  double Cm[6][6], Sm[6];
  gauss_elasticity(law, c, Fm, J, p, Cm, Sm);
  for (int i = 0; i < 6; ++i) {
    if (C)
      for (int j = 0; j < 6; ++j) C[i * 6 + j] = Cm[i][j];
  }
  double S2[6];
  gauss_stress(law, c, Fm, J, p, S2);
  for (int i = 0; i < 6; ++i) S[i] = S2[i];
}

}  // extern "C"
