// libcm_fe: the Jacobian's CSR sparsity pattern built on the GPU (sm_103a).
//
// Same rule as the host set-up (and as JacobianMatrix_StructureCalculate,
// equations_matrices_routines.f90:5048-5340): the row of a dof at row node R
// (a u node for displacement rows, a pressure node -- or the element itself
// for element-based pressure -- for pressure rows) holds, in this order,
// the u_x, u_y and u_z dofs of every u node of the elements around R, then
// the pressure dofs of those elements, each list sorted and without repeats.
//
//   1. count the elements around every row node, scan, fill, sort each list;
//   2. one warp per row node gathers the candidate nodes of its elements into
//      shared memory, sorts them (bitonic) and keeps the first of each run --
//      once to count, once (after a scan) to write;
//   3. row lengths 3*|U| + |P| are scanned into row_ptr and one warp per row
//      writes its columns.
// Every step is deterministic (sorted lists, fixed write positions).
#include <cuda_runtime.h>

#include <climits>
#include <cstdint>
#include <string>
#include <vector>

#include "cm_fe.h"
#include "fe_internal.h"

namespace {

constexpr int WARPS = 8;
constexpr int CAND = 512;  // candidate slots per warp (8 elements x 27 nodes = 216 on hexahedral boxes)

__global__ void count_kernel(const int32_t* __restrict__ en, int64_t n, int32_t* cnt) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    atomicAdd(&cnt[en[i]], 1);
}

__global__ void fill_kernel(const int32_t* __restrict__ en, int64_t n, int per, const int32_t* off, int32_t* cur,
                            int32_t* adj) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t node = en[i];
    const int32_t k = atomicAdd(&cur[node], 1);
    adj[off[node] + k] = (int32_t)(i / per);  // element number
  }
}

// Element lists of one row node in ascending order (they are short).
__global__ void sort_lists_kernel(const int32_t* off, int32_t n, int32_t* adj) {
  for (int32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    const int32_t a = off[v], b = off[v + 1];
    for (int32_t i = a + 1; i < b; ++i) {
      const int32_t x = adj[i];
      int32_t j = i - 1;
      while (j >= a && adj[j] > x) {
        adj[j + 1] = adj[j];
        --j;
      }
      adj[j + 1] = x;
    }
  }
}

// Exclusive scan of n values in one CTA (per node or per row counts: a few
// million at most); out has n + 1 entries, out[n] the total.  With w given,
// the values are the row lengths 3 |U| + |P| of the n dofs, w holding
// (|U|, |P|) per row node (u nodes, then pressure row nodes).
__global__ void __launch_bounds__(1024) scan_kernel(const int32_t* in, int64_t n, int64_t* out, int64_t nu,
                                                    const int32_t* w) {
  __shared__ int64_t part[1024];
  const int t = threadIdx.x;
  const int64_t chunk = (n + 1023) / 1024;
  const int64_t a = t * chunk, b = a + chunk < n ? a + chunk : n;
  auto val = [&](int64_t i) -> int64_t {
    if (!w) return in[i];
    const int64_t v = i < 3 * nu ? i % nu : nu + (i - 3 * nu);
    return 3ll * w[2 * v] + w[2 * v + 1];
  };
  int64_t s = 0;
  for (int64_t i = a; i < b; ++i) s += val(i);
  part[t] = s;
  __syncthreads();
  if (t == 0) {
    int64_t run = 0;
    for (int i = 0; i < 1024; ++i) {
      const int64_t v = part[i];
      part[i] = run;
      run += v;
    }
    out[n] = run;
  }
  __syncthreads();
  int64_t run = part[t];
  for (int64_t i = a; i < b; ++i) {
    out[i] = run;
    run += val(i);
  }
}

__global__ void to_int32_kernel(const int64_t* in, int64_t n, int32_t* out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (int32_t)in[i];
}

struct NbArgs {
  const int32_t* elem_u;  // [ne][npe]
  const int32_t* elem_p;  // [ne][8], or NULL for element-based pressure (the element itself)
  int npe, npp;
  const int32_t* off_u;   // elements around u nodes
  const int32_t* adj_u;
  const int32_t* off_p;   // elements around pressure row nodes
  const int32_t* adj_p;
  int32_t nu, npn;
  int32_t* w;             // [nu + npn][2]: |U|, |P| per row node (count pass)
  const int64_t* nb_off;  // [nu + npn][2] output offsets (write pass), NULL in the count pass
  int32_t* nb;            // neighbour lists (write pass)
  unsigned* status;       // bit 0: a row node has more than CAND candidates
};

__device__ int sort_unique_warp(int32_t* buf, int n, int lane) {
  for (int i = n + lane; i < CAND; i += 32) buf[i] = INT_MAX;
  __syncwarp();
  for (int k = 2; k <= CAND; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = lane; i < CAND; i += 32) {
        const int l = i ^ j;
        if (l > i) {
          const int32_t x = buf[i], y = buf[l];
          const bool up = (i & k) == 0;
          if ((x > y) == up) {
            buf[i] = y;
            buf[l] = x;
          }
        }
      }
      __syncwarp();
    }
  // Compact the first of each run in place (ballot prefix over chunks of 32).
  // The predecessor of each value comes from registers (shuffle, and the last
  // value of the previous chunk carried over), never from the part of the
  // buffer already overwritten.
  int outn = 0;
  int32_t carry = INT_MIN;
  for (int base = 0; base < CAND; base += 32) {
    const int32_t v = buf[base + lane];
    int32_t prev = __shfl_up_sync(0xffffffffu, v, 1);
    if (lane == 0) prev = carry;
    carry = __shfl_sync(0xffffffffu, v, 31);
    const bool keep = v != INT_MAX && v != prev;
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    __syncwarp();
    if (keep) buf[outn + __popc(m & ((1u << lane) - 1))] = v;
    __syncwarp();
    outn += __popc(m);
  }
  return outn;
}

__global__ void __launch_bounds__(32 * WARPS) neighbours_kernel(NbArgs A) {
  __shared__ int32_t sbuf[WARPS][CAND];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int32_t* buf = sbuf[warp];
  const int32_t nrow = A.nu + A.npn;
  for (int32_t v = blockIdx.x * WARPS + warp; v < nrow; v += gridDim.x * WARPS) {
    const bool unode = v < A.nu;
    const int32_t* off = unode ? A.off_u : A.off_p;
    const int32_t* adj = unode ? A.adj_u : A.adj_p;
    const int32_t node = unode ? v : v - A.nu;
    const int32_t a = off[node], b = off[node + 1];
    for (int pass = 0; pass < 2; ++pass) {  // 0: u nodes, 1: pressure row nodes
      const int per = pass == 0 ? A.npe : A.npp;
      const int n = (b - a) * per;
      if (n > CAND) {
        if (lane == 0) atomicOr(A.status, 1u);
        continue;
      }
      for (int i = lane; i < n; i += 32) {
        const int32_t e = adj[a + i / per], k = i % per;
        buf[i] = pass == 0 ? A.elem_u[(int64_t)e * A.npe + k] : (A.elem_p ? A.elem_p[(int64_t)e * 8 + k] : e);
      }
      __syncwarp();
      const int m = sort_unique_warp(buf, n, lane);
      if (!A.nb_off) {
        if (lane == 0) A.w[2 * v + pass] = m;
      } else {
        const int64_t o = A.nb_off[2 * v + pass];
        for (int i = lane; i < m; i += 32) A.nb[o + i] = buf[i];
      }
      __syncwarp();
    }
  }
}

__global__ void columns_kernel(const int64_t* row_ptr, int64_t nrows, int32_t nu, const int64_t* nb_off,
                               const int32_t* w, const int32_t* nb, int32_t base, int32_t* col) {
  const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = warp; r < nrows; r += nwarps) {
    const int64_t v = r < 3ll * nu ? r % nu : nu + (r - 3ll * nu);
    const int32_t wu = w[2 * v], wp = w[2 * v + 1];
    const int32_t* U = nb + nb_off[2 * v];
    const int32_t* Pn = nb + nb_off[2 * v + 1];
    int32_t* out = col + row_ptr[r];
    for (int i = lane; i < 3 * wu; i += 32) out[i] = (i / wu) * nu + U[i % wu] + base;
    for (int i = lane; i < wp; i += 32) out[3 * wu + i] = 3 * nu + Pn[i] + base;
  }
}

int grid_for(int64_t n, int per = 256) {
  const int64_t g = (n + per - 1) / per;
  return (int)(g < 8192 ? (g < 1 ? 1 : g) : 8192);
}

struct DevBuf {
  std::vector<void*> ptrs;
  ~DevBuf() {
    for (void* p : ptrs) cudaFree(p);
  }
  template <class T>
  cudaError_t get(T** p, size_t count) {
    *p = nullptr;
    if (count == 0) count = 1;
    const cudaError_t e = cudaMalloc((void**)p, count * sizeof(T));
    if (e == cudaSuccess) ptrs.push_back(*p);
    return e;
  }
};

}  // namespace

extern "C" int fe_structure_calculate_device(const fe_mesh_desc* d, int32_t base, int64_t* num_dofs, int64_t* nnz,
                                             int32_t* row_ptr, int32_t* col, void* stream) {
  if (!d || (base != 0 && base != 1)) return cmfe::record_error(FE_ERR_INVALID_ARGUMENT, "bad descriptor or base");
  if (d->num_elements <= 0 || d->num_nodes_u <= 0 || (d->nodes_per_xi_u != 2 && d->nodes_per_xi_u != 3) ||
      !d->element_nodes_u)
    return cmfe::record_error(FE_ERR_INVALID_ARGUMENT, "invalid mesh description");
  const bool pm = d->pressure_interpolation == FE_PRESSURE_NODE_BASED;
  if (pm && (!d->element_nodes_p || d->num_nodes_p <= 0))
    return cmfe::record_error(FE_ERR_INVALID_ARGUMENT, "node-based pressure needs element_nodes_p and num_nodes_p");
  const int32_t ne = d->num_elements, nu = d->num_nodes_u, n1 = d->nodes_per_xi_u;
  const int npe = n1 * n1 * n1, npp = pm ? 8 : 1;
  const int32_t npn = pm ? d->num_nodes_p : ne;
  const int64_t ndofs = 3ll * nu + npn;
  if (ndofs >= (1ll << 31)) return cmfe::record_error(FE_ERR_INVALID_ARGUMENT, "too many dofs for 32-bit CSR indices");
  for (int64_t i = 0; i < (int64_t)ne * npe; ++i)
    if (d->element_nodes_u[i] < 0 || d->element_nodes_u[i] >= nu)
      return cmfe::record_error(FE_ERR_INVALID_ARGUMENT, "element_nodes_u entry out of range");
  if (pm)
    for (int64_t i = 0; i < (int64_t)ne * 8; ++i)
      if (d->element_nodes_p[i] < 0 || d->element_nodes_p[i] >= npn)
        return cmfe::record_error(FE_ERR_INVALID_ARGUMENT, "element_nodes_p entry out of range");
  cudaStream_t st = (cudaStream_t)stream;
  DevBuf mem;
  auto fail = [&](cudaError_t e, const char* what) {
    return cmfe::record_error(FE_ERR_CUDA, std::string("device pattern: ") + what + ": " + cudaGetErrorString(e));
  };
#define PT_TRY(expr, what)                          \
  do {                                              \
    const cudaError_t e__ = (expr);                 \
    if (e__ != cudaSuccess) return fail(e__, what); \
  } while (0)
  int32_t *eu = nullptr, *ep = nullptr, *pnodes = nullptr, *cnt_u, *cnt_p, *cur_u, *cur_p, *adj_u, *adj_p, *w,
          *nb = nullptr, *off_u, *off_p;
  int64_t *off_u64, *off_p64, *nb_off, *rp64;
  unsigned* status;
  PT_TRY(mem.get(&eu, (size_t)ne * npe), "allocation");
  PT_TRY(cudaMemcpyAsync(eu, d->element_nodes_u, sizeof(int32_t) * ne * npe, cudaMemcpyHostToDevice, st), "copy");
  std::vector<int32_t> self;
  if (pm) {
    PT_TRY(mem.get(&ep, (size_t)ne * 8), "allocation");
    PT_TRY(cudaMemcpyAsync(ep, d->element_nodes_p, sizeof(int32_t) * ne * 8, cudaMemcpyHostToDevice, st), "copy");
    pnodes = ep;
  } else {  // element-based pressure: the pressure row node of element e is e
    self.resize(ne);
    for (int32_t e = 0; e < ne; ++e) self[e] = e;
    PT_TRY(mem.get(&pnodes, ne), "allocation");
    PT_TRY(cudaMemcpyAsync(pnodes, self.data(), sizeof(int32_t) * ne, cudaMemcpyHostToDevice, st), "copy");
  }
  PT_TRY(mem.get(&cnt_u, nu), "allocation");
  PT_TRY(mem.get(&cnt_p, npn), "allocation");
  PT_TRY(mem.get(&cur_u, nu), "allocation");
  PT_TRY(mem.get(&cur_p, npn), "allocation");
  PT_TRY(mem.get(&off_u64, (size_t)nu + 1), "allocation");
  PT_TRY(mem.get(&off_p64, (size_t)npn + 1), "allocation");
  PT_TRY(mem.get(&off_u, (size_t)nu + 1), "allocation");
  PT_TRY(mem.get(&off_p, (size_t)npn + 1), "allocation");
  PT_TRY(mem.get(&adj_u, (size_t)ne * npe), "allocation");
  PT_TRY(mem.get(&adj_p, (size_t)ne * npp), "allocation");
  PT_TRY(mem.get(&w, 2ull * (nu + npn)), "allocation");
  PT_TRY(mem.get(&nb_off, 2ull * (nu + npn) + 1), "allocation");
  PT_TRY(mem.get(&rp64, (size_t)ndofs + 1), "allocation");
  PT_TRY(mem.get(&status, 1), "allocation");
  PT_TRY(cudaMemsetAsync(cnt_u, 0, sizeof(int32_t) * nu, st), "memset");
  PT_TRY(cudaMemsetAsync(cnt_p, 0, sizeof(int32_t) * npn, st), "memset");
  PT_TRY(cudaMemsetAsync(cur_u, 0, sizeof(int32_t) * nu, st), "memset");
  PT_TRY(cudaMemsetAsync(cur_p, 0, sizeof(int32_t) * npn, st), "memset");
  PT_TRY(cudaMemsetAsync(status, 0, sizeof(unsigned), st), "memset");
  const int64_t nu_e = (int64_t)ne * npe, np_e = (int64_t)ne * npp;
  count_kernel<<<grid_for(nu_e), 256, 0, st>>>(eu, nu_e, cnt_u);
  count_kernel<<<grid_for(np_e), 256, 0, st>>>(pnodes, np_e, cnt_p);
  scan_kernel<<<1, 1024, 0, st>>>(cnt_u, nu, off_u64, 0, nullptr);
  scan_kernel<<<1, 1024, 0, st>>>(cnt_p, npn, off_p64, 0, nullptr);
  to_int32_kernel<<<grid_for((int64_t)nu + 1), 256, 0, st>>>(off_u64, (int64_t)nu + 1, off_u);
  to_int32_kernel<<<grid_for((int64_t)npn + 1), 256, 0, st>>>(off_p64, (int64_t)npn + 1, off_p);
  fill_kernel<<<grid_for(nu_e), 256, 0, st>>>(eu, nu_e, npe, off_u, cur_u, adj_u);
  fill_kernel<<<grid_for(np_e), 256, 0, st>>>(pnodes, np_e, npp, off_p, cur_p, adj_p);
  sort_lists_kernel<<<grid_for(nu), 256, 0, st>>>(off_u, nu, adj_u);
  sort_lists_kernel<<<grid_for(npn), 256, 0, st>>>(off_p, npn, adj_p);
  NbArgs A;
  A.elem_u = eu;
  A.elem_p = ep;
  A.npe = npe;
  A.npp = npp;
  A.off_u = off_u;
  A.adj_u = adj_u;
  A.off_p = off_p;
  A.adj_p = adj_p;
  A.nu = nu;
  A.npn = npn;
  A.w = w;
  A.nb_off = nullptr;
  A.nb = nullptr;
  A.status = status;
  const int nb_grid = grid_for((int64_t)nu + npn, WARPS);
  neighbours_kernel<<<nb_grid, 32 * WARPS, 0, st>>>(A);
  scan_kernel<<<1, 1024, 0, st>>>(w, 2ll * (nu + npn), nb_off, 0, nullptr);
  int64_t nb_total = 0;
  unsigned stat = 0;
  PT_TRY(cudaMemcpyAsync(&nb_total, nb_off + 2ll * (nu + npn), sizeof(int64_t), cudaMemcpyDeviceToHost, st), "copy");
  PT_TRY(cudaMemcpyAsync(&stat, status, sizeof(unsigned), cudaMemcpyDeviceToHost, st), "copy");
  PT_TRY(cudaStreamSynchronize(st), "synchronise");
  PT_TRY(cudaGetLastError(), "kernel launch");
  if (stat & 1u)
    return cmfe::record_error(FE_ERR_NOT_SUPPORTED, "a row node has more than 512 candidate neighbour nodes");
  PT_TRY(mem.get(&nb, (size_t)nb_total), "allocation");
  A.nb_off = nb_off;
  A.nb = nb;
  neighbours_kernel<<<nb_grid, 32 * WARPS, 0, st>>>(A);
  scan_kernel<<<1, 1024, 0, st>>>(nullptr, ndofs, rp64, nu, w);
  int64_t total = 0;
  PT_TRY(cudaMemcpyAsync(&total, rp64 + ndofs, sizeof(int64_t), cudaMemcpyDeviceToHost, st), "copy");
  PT_TRY(cudaStreamSynchronize(st), "synchronise");
  PT_TRY(cudaGetLastError(), "kernel launch");
  if (total >= (1ll << 31)) return cmfe::record_error(FE_ERR_INVALID_ARGUMENT, "too many nonzeros for 32-bit CSR indices");
  if (num_dofs) *num_dofs = ndofs;
  if (nnz) *nnz = total;
  if (row_ptr) {
    std::vector<int64_t> h(ndofs + 1);
    PT_TRY(cudaMemcpyAsync(h.data(), rp64, sizeof(int64_t) * (ndofs + 1), cudaMemcpyDeviceToHost, st), "copy");
    PT_TRY(cudaStreamSynchronize(st), "synchronise");
    std::vector<int32_t> h32(ndofs + 1);
    for (int64_t i = 0; i <= ndofs; ++i) h32[i] = (int32_t)h[i] + base;
    PT_TRY(cudaMemcpyAsync(row_ptr, h32.data(), sizeof(int32_t) * (ndofs + 1), cudaMemcpyDefault, st), "copy");
    PT_TRY(cudaStreamSynchronize(st), "synchronise");
  }
  if (col) {
    int32_t* dcol = nullptr;
    PT_TRY(mem.get(&dcol, (size_t)total), "allocation");
    columns_kernel<<<grid_for(ndofs * 32), 256, 0, st>>>(rp64, ndofs, nu, nb_off, w, nb, base, dcol);
    PT_TRY(cudaMemcpyAsync(col, dcol, sizeof(int32_t) * total, cudaMemcpyDefault, st), "copy");
  }
  PT_TRY(cudaStreamSynchronize(st), "synchronise");
  PT_TRY(cudaGetLastError(), "kernel launch");
  return FE_NO_ERROR;
#undef PT_TRY
}
