// Internal declarations shared by the host set-up (fe_setup.cpp) and the
// device code / C ABI (fe_kernels.cu) of libcm_fe.
#pragma once
#include <cstddef>
#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "../../include/cm_fe.h"

namespace cmfe {

constexpr int NG = 27;  // 3x3x3 Gauss-Legendre points per element

// Growable-once array without value initialisation (large index arrays are
// first touched by the threads that fill them).
template <class T>
struct RawArray {
  std::shared_ptr<T[]> p;  // shared by copies (handles cloned from one set-up)
  size_t n = 0;
  void allocate(size_t count) {
    p.reset(new T[count]);
    n = count;
  }
  T* data() { return p.get(); }
  const T* data() const { return p.get(); }
  size_t size() const { return n; }
  T& operator[](size_t i) { return p[i]; }
  const T& operator[](size_t i) const { return p[i]; }
};

// Everything the device kernels need, built once on the host by fe_create.
struct HostSetup {
  int ne = 0, nu = 0, npn = 0;  // elements, u nodes, pressure "row nodes" (p nodes or elements)
  int n1 = 0, npe = 0, npp = 0; // u nodes per xi, u params per element, p params per element
  int nr = 0;                   // local row nodes per element: npe + npp
  int nrow = 0;                 // element dofs: 3*npe + npp
  int pmode = 0, law = 0, nmat = 0, mat_per_element = 0;
  bool fibre = false;
  int64_t ndofs = 0, nnz = 0, nnz_uu = 0, nnz_cp = 0;

  std::vector<int32_t> elem_u, elem_p;   // connectivity (elem_p empty for element-based p)
  std::vector<double> mat;               // materials
  std::vector<int32_t> row_ptr;          // 0-based CSR pattern
  RawArray<int32_t> col;
  std::vector<int32_t> uu_row_ptr, cp_row_ptr;
  std::vector<int32_t> wu, wp;           // u-node count of the u-column block of a node's rows
  int ncolours = 0;
  std::vector<int32_t> colour_ptr, colour_elems;
  int ntables = 0;
  std::vector<uint16_t> tables;          // [ntables][nr][nr]: CSR rank | first-contributor bit 15
  std::vector<int32_t> elem_table;       // [ne]
  std::vector<double> geo;               // [ne][NG][10]: dXi/dNu (row-major) and J_x
  std::vector<double> gbf_u, gbf_p, gw;  // quadrature tables
  // elements with at least one boundary face, grouped by colour, and a mask of
  // their boundary local faces (reference local-face order)
  std::vector<int32_t> bnd_elems, bnd_ptr;
  std::vector<uint8_t> bnd_mask;
  // Row-node incidence for the staged assembly: the elements around every u
  // node (sorted by element number, packed e * 32 + local node) and around
  // every pressure row node (e * 8 + local pressure node).
  std::vector<int32_t> u_inc_ptr, u_inc, p_inc_ptr, p_inc;
  // the largest element number around any of the row nodes 0..a (u nodes)
  // and 0..q (pressure row nodes): once the elements below E are assembled,
  // every node a with u_last_prefix[a] < E has its rows complete
  std::vector<int32_t> u_last_prefix, p_last_prefix;
  // shared memory one gather warp needs: the larger of a u node's three rows
  // (3 x 3 wu FP32, then 3 x its pressure columns FP64) and a pressure row (FP64)
  int gather_bytes = 0;
};

// Arguments of the element kernels (plain data; device pointers).
struct KParams {
  int nu, law, nmat, matpe;
  const int32_t* elem_u;
  const int32_t* elem_p;
  const double* geo;
  const float* geo_dd;  // geo as (hi, lo) FP32 pairs, for the double-float variant
  const double* mat;
  const double* gbf_u;
  const double* gbf_p;
  const double* gw;
  const int32_t* row_ptr;
  const int32_t* uu_row_ptr;
  const int32_t* cp_row_ptr;
  const int32_t* wu;
  const int32_t* wp;
  const uint16_t* tables;
  const int32_t* elem_table;
  const int32_t* elems;  // element list of this launch (NULL: first_elem + i)
  int count;
  int first_elem;
  const double* x;
  double* r;
  double* vals;      // FP64 CSR values, or FP64 coupling values (mixed)
  float* vals_uu;    // FP32 uu values (mixed)
  double* elem_out;  // element-level output
  int res_only;      // mixed kernel: residual only (no Jacobian blocks)
  int wave;          // mixed kernel: CTAs per launch wave (the SM count)
  int nr, pmode;     // local row nodes per element, pressure interpolation
  const double* surf_p;  // surface pressure values [3][nu] (surface kernel)
  unsigned* status;
};

#ifdef __CUDACC__
#define CMFE_HD __host__ __device__
#else
#define CMFE_HD
#endif

// Strides of the per-element records of the staged assembly, in elements of
// each record's type, rounded up to whole 128-byte lines, so that no L2 line
// holds parts of two elements' records (npe u nodes and npp pressure
// parameters per element).
CMFE_HD constexpr int rec_stride_uu(int npe) { return (9 * npe * npe + 31) / 32 * 32; }          // floats
CMFE_HD constexpr int rec_stride_cp(int npe, int npp) { return (npp * 3 * npe + 15) / 16 * 16; }  // doubles
CMFE_HD constexpr int rec_stride_r(int npe, int npp) { return (3 * npe + npp + 15) / 16 * 16; }   // doubles

// Per-element records of the staged assembly (mixed kernel with staged
// output, surface mode 2, row gather): the full displacement block
// [3 NPE][3 NPE] (FP32, row-major), the pressure-coupling rows [NPP][3 NPE]
// and the residual [nrow] (FP64) of element e, at e times the strides above.
struct StageOut {
  float* uu;
  double* cp;
  double* r;
};

// Arguments of the fused staged assembly (fe_mixed.cu): the incidence lists,
// a work counter (next element group, zero before the launch), the per-row-
// node counts of finished elements around the node (u nodes, then pressure
// row nodes; zero before the launch), and the boundary-face masks when a
// surface-pressure load is set (else NULL).
struct FusedArgs {
  const int32_t* u_inc_ptr;
  const int32_t* u_inc;
  const int32_t* p_inc_ptr;
  const int32_t* p_inc;
  int* work;       // this launch's group counter
  int* node_done;
  const uint8_t* bmask;
  int g0, g1;      // element groups of this launch: [g0, g1)
  int gwarps;  // warps that gather (set by the launcher)
  int gbytes;  // scratch bytes per gathering warp (set by the launcher)
};

// Launches the mixed-precision assembly kernel for one colour (fe_mixed.cu),
// with the high-precision phases in FP64 or in double-float arithmetic.
// Returns a cudaError_t value.
int launch_mixed(const HostSetup& s, const KParams& kp, int num_sms, void* stream, bool double_float);

// Elements per group of the fused kernel for this element type.
int fused_group_size(const HostSetup& s);

// Blocks of the fused kernel resident on the whole GPU at once (the groups
// one wave of the launch takes); a negative cudaError_t on failure.
int fused_wave(const HostSetup& s, int num_sms, bool double_float);

// Launches the mixed-precision assembly kernel over all elements with its
// output staged per element (so; fe_mixed.cu), in
// one launch, without colour order.  Returns a cudaError_t value.
int launch_mixed_staged(const HostSetup& s, const KParams& kp, const StageOut& so, int num_sms, void* stream,
                        bool double_float);

// The staged assembly in one launch with the row gathers inside it
// (fe_mixed.cu); fused_fits() says whether a mesh's largest row node fits the
// kernel's gather scratch.  Returns a cudaError_t value.
int fused_fits(const HostSetup& s);
int launch_mixed_fused(const HostSetup& s, const KParams& kp, const StageOut& so, const FusedArgs& fa, int num_sms,
                       void* stream, bool double_float);

// Sums the staged element outputs into the CSR rows (uu FP32, coupling FP64)
// and the residual, one row node at a time, in the fixed element order of
// the incidence lists (fe_gather.cu).  Returns a cudaError_t value.
int launch_gather(const HostSetup& s, const KParams& kp, const StageOut& so, const int32_t* u_inc_ptr,
                  const int32_t* u_inc, const int32_t* p_inc_ptr, const int32_t* p_inc, int num_sms, void* stream);

// Launches the surface-pressure kernel over boundary elements (fe_surface.cu):
// mode 0 adds into the CSR values / residual, mode 1 into element outputs,
// mode 2 into the staged element records (so.uu, so.r).
// Returns a cudaError_t value.
int launch_surface(const HostSetup& s, const KParams& kp, const int32_t* belems, const uint8_t* bmask, int nb,
                   int mode, int want_jac, int num_sms, void* stream, const StageOut& so = StageOut{});

// Builds the set-up; returns FE_NO_ERROR or a FE_ERR_* code with msg filled.
int build_setup(const fe_mesh_desc* d, HostSetup& s, std::string& msg);

// Batched mixed assembly (fe_batch.cu).  The members' parameters live in a
// constant-memory table of the batch module, one entry per member slot
// (slots ordered by element type), so that the persistent kernel reads them
// as warp-uniform operands, as the single-set kernels read their launch
// parameters.
constexpr int BATCH_MAX_MEMBERS = 256;

struct BatchMember {
  KParams kp;                // elems: the member's colour-ordered element list; x, r, vals, vals_uu of the call
  const int32_t* belems;     // boundary elements grouped by colour
  const uint8_t* bmask;      // boundary faces per element
  int type;                  // 2 * (N1 == 3) + nodal pressure
  int has_surface;           // surface-pressure load set (kp.surf_p)
};

struct BatchArgs {
  const int32_t* offsets;    // [slot][2][ncolours + 1]: colour element offsets, then boundary element offsets
  int nmembers;
  int ncolours;
  int block_groups;          // consecutive element groups per work unit
  int wave;                  // CTAs per launch wave (the SM count)
  unsigned* bar_count;       // grid barrier state (zero before a launch)
  unsigned* bar_gen;
  unsigned* status;          // bit 1: a grid barrier gave up waiting
  unsigned barrier_polls;    // polls before a barrier gives up (0: the default limit)
  unsigned barrier_extra;    // arrivals a barrier waits for beyond the grid (0; a diagnostic sets
                             // 1 to make every barrier give up and report)
};

// Number of launch variants, their elements per group (triquadratic,
// trilinear) and dynamic shared memory for the element types present (mask
// bit t = type t, bit 4 = surface loads).
int batch_variants();
int batch_variant_eg(int v, int* egq, int* egl);
int batch_smem(int v, unsigned mask);
// Copies the member table (device memory, n entries) into the constant table
// and launches the persistent kernel, both on stream; returns a cudaError_t.
int launch_mixed_batch(int variant, unsigned mask, const BatchMember* members, int n, const BatchArgs& a,
                       int ctas_per_sm, int num_sms, void* stream);
// The same for a batch whose members all have element type `type`
// (fe_batch_typed.cu).
int launch_batch_typed(int variant, int type, unsigned mask, const BatchMember* members, int n, const BatchArgs& a,
                       int ctas_per_sm, int num_sms, void* stream);

// Device CSR pattern (0-based row pointers and columns) and sizes of a handle
// (fe_kernels.cu), for the Newton driver (fe_newton.cu).
int device_pattern(fe_handle h, const int32_t** row_ptr, const int32_t** col, int64_t* ndofs, int64_t* nnz,
                   int64_t* nu3);

// Records the text fe_last_error() returns (per calling thread) and returns code.
int record_error(int code, const std::string& msg);

}  // namespace cmfe
