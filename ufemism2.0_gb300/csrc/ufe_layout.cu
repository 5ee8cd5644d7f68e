// Internal memory layout of a mesh: vertices and triangles are renumbered along a Z-order
// (Morton) curve of their coordinates, so that neighbours in the mesh sit close together in
// memory and the gathers of the operator, assembly and Krylov kernels hit the same cache lines.
//
// Internal index i holds the caller's index perm[i]; iperm is the inverse.  Every array that
// crosses the C ABI is mapped here: inputs are gathered into internal order, outputs gathered
// back into the caller's order.  The mapping is a pure relabelling -- each operator row keeps
// its entries in the reference's order -- so exported matrices are identical to what the
// reference builds for the caller's numbering.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <numeric>

#include "ufe_internal.cuh"

namespace {

uint64_t spread_bits(uint32_t v) {
  uint64_t x = v & 0x1fffff;   // 21 bits
  x = (x | (x << 32)) & 0x1f00000000ffffull;
  x = (x | (x << 16)) & 0x1f0000ff0000ffull;
  x = (x | (x << 8)) & 0x100f00f00f00f00full;
  x = (x | (x << 4)) & 0x10c30c30c30c30c3ull;
  x = (x | (x << 2)) & 0x1249249249249249ull;
  return x;
}

std::vector<int32_t> morton_order(const double *x, const double *y, int64_t n, bool identity) {
  std::vector<int32_t> idx(n);
  std::iota(idx.begin(), idx.end(), 0);
  if (identity || n < 2) return idx;
  double x0 = x[0], x1 = x[0], y0 = y[0], y1 = y[0];
  for (int64_t i = 1; i < n; ++i) {
    x0 = std::min(x0, x[i]); x1 = std::max(x1, x[i]);
    y0 = std::min(y0, y[i]); y1 = std::max(y1, y[i]);
  }
  const double sx = (x1 > x0) ? 2097151.0 / (x1 - x0) : 0.0, sy = (y1 > y0) ? 2097151.0 / (y1 - y0) : 0.0;
  std::vector<uint64_t> code(n);
  for (int64_t i = 0; i < n; ++i) {
    uint32_t ix = (uint32_t)((x[i] - x0) * sx), iy = (uint32_t)((y[i] - y0) * sy);
    code[i] = spread_bits(ix) | (spread_bits(iy) << 1);
  }
  std::stable_sort(idx.begin(), idx.end(), [&](int32_t a, int32_t b) { return code[a] < code[b]; });
  return idx;
}

template <class T>
T *upload_vec(const std::vector<T> &h, cudaStream_t s) {
  T *d = (T *)dev_alloc(sizeof(T) * (h.empty() ? 1 : h.size()));
  if (!h.empty()) UFE_CUDA(cudaMemcpyAsync(d, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice, s));
  return d;
}

// dst[c*n + i] = src[c*n + map[i]]
template <class T>
__global__ void k_gather_cols(int64_t n, int ncols, const T *__restrict__ src, const int32_t *__restrict__ map,
                              T *__restrict__ dst) {
  int64_t total = n * ncols;
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += stride) {
    int64_t c = e / n, i = e - c * n;
    dst[e] = src[c * n + map[i]];
  }
}

// out[i] = (a[map[i]], b[map[i]])
__global__ void k_gather_pair(int64_t n, const double *a, const double *b, const int32_t *map, double2 *out) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    int32_t j = map[i];
    out[i] = make_double2(a ? a[j] : 0.0, b ? b[j] : 0.0);
  }
}

// a[j] = in[map[j]].x, b[j] = in[map[j]].y
__global__ void k_scatter_pair(int64_t n, const double2 *in, const int32_t *map, double *a, double *b) {
  int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += stride) {
    double2 w = in[map[j]];
    a[j] = w.x;
    b[j] = w.y;
  }
}

int blocks_for(int64_t n) {
  int64_t b = (n + 255) / 256;
  return (int)std::max<int64_t>(1, std::min<int64_t>(b, 4096));
}

}  // namespace

void free_layout(ufe_ctx *ctx) {
  dev_free(ctx->perm_v); dev_free(ctx->iperm_v); dev_free(ctx->perm_t); dev_free(ctx->iperm_t);
  ctx->perm_v = ctx->iperm_v = ctx->perm_t = ctx->iperm_t = nullptr;
  ctx->perm_v_h.clear(); ctx->iperm_v_h.clear(); ctx->perm_t_h.clear(); ctx->iperm_t_h.clear();
}

// Renumber the mesh and upload it in internal order.
void layout_upload_mesh(ufe_ctx *ctx, const ufe_mesh_desc *m) {
  const int64_t nV = m->nV, nTri = m->nTri, nCm = m->nC_mem;
  const char *e = getenv("UFE_NO_REORDER");
  const bool identity = e && *e && *e != '0';
  cudaStream_t s = ctx->stream;
  ctx->perm_v_h = morton_order(m->V, m->V + nV, nV, identity);
  ctx->perm_t_h = morton_order(m->TriGC, m->TriGC + nTri, nTri, identity);
  ctx->iperm_v_h.assign(nV, 0);
  ctx->iperm_t_h.assign(nTri, 0);
  for (int64_t i = 0; i < nV; ++i) ctx->iperm_v_h[ctx->perm_v_h[i]] = (int32_t)i;
  for (int64_t i = 0; i < nTri; ++i) ctx->iperm_t_h[ctx->perm_t_h[i]] = (int32_t)i;
  const auto &pv = ctx->perm_v_h, &iv = ctx->iperm_v_h, &pt = ctx->perm_t_h, &it = ctx->iperm_t_h;
  auto vmap = [&](int32_t v1) { return v1 == 0 ? 0 : iv[v1 - 1] + 1; };   // 1-based renumbering
  auto tmap = [&](int32_t t1) { return t1 == 0 ? 0 : it[t1 - 1] + 1; };
  std::vector<double> V(2 * nV), TriGC(2 * nTri);
  std::vector<int32_t> nC(nV), C(nV * nCm), niTri(nV), iTri(nV * nCm), VBI(nV);
  std::vector<int32_t> Tri(3 * nTri), TriC(3 * nTri), TriBI(nTri);
  for (int64_t i = 0; i < nV; ++i) {
    const int64_t o = pv[i];
    V[i] = m->V[o];
    V[nV + i] = m->V[nV + o];
    nC[i] = m->nC[o];
    niTri[i] = m->niTri[o];
    VBI[i] = m->VBI[o];
    for (int64_t c = 0; c < nCm; ++c) {
      C[c * nV + i] = vmap(m->C[c * nV + o]);
      iTri[c * nV + i] = tmap(m->iTri[c * nV + o]);
    }
  }
  for (int64_t t = 0; t < nTri; ++t) {
    const int64_t o = pt[t];
    TriGC[t] = m->TriGC[o];
    TriGC[nTri + t] = m->TriGC[nTri + o];
    TriBI[t] = m->TriBI[o];
    for (int n = 0; n < 3; ++n) {
      Tri[n * nTri + t] = vmap(m->Tri[n * nTri + o]);
      TriC[n * nTri + t] = tmap(m->TriC[n * nTri + o]);
    }
  }
  ctx->V = upload_vec(V, s);
  ctx->nC = upload_vec(nC, s);
  ctx->C = upload_vec(C, s);
  ctx->niTri = upload_vec(niTri, s);
  ctx->iTri = upload_vec(iTri, s);
  ctx->VBI = upload_vec(VBI, s);
  ctx->Tri = upload_vec(Tri, s);
  ctx->TriC = upload_vec(TriC, s);
  ctx->TriBI = upload_vec(TriBI, s);
  ctx->TriGC = upload_vec(TriGC, s);
  ctx->perm_v = upload_vec(ctx->perm_v_h, s);
  ctx->iperm_v = upload_vec(ctx->iperm_v_h, s);
  ctx->perm_t = upload_vec(ctx->perm_t_h, s);
  ctx->iperm_t = upload_vec(ctx->iperm_t_h, s);
  UFE_CUDA(cudaStreamSynchronize(s));
}

const int32_t *perm_of(ufe_ctx *ctx, bool tri) { return tri ? ctx->perm_t : ctx->perm_v; }
const int32_t *iperm_of(ufe_ctx *ctx, bool tri) { return tri ? ctx->iperm_t : ctx->iperm_v; }

template <class T>
void to_internal_t(ufe_ctx *ctx, T *d_dst, const T *h_src, bool tri, int ncols) {
  const int64_t n = tri ? ctx->nTri : ctx->nV;
  cudaStream_t s = ctx->stream;
  T *tmp = (T *)dev_alloc(sizeof(T) * n * ncols);
  UFE_CUDA(cudaMemcpyAsync(tmp, h_src, sizeof(T) * n * ncols, cudaMemcpyHostToDevice, s));
  k_gather_cols<T><<<blocks_for(n * ncols), 256, 0, s>>>(n, ncols, tmp, perm_of(ctx, tri), d_dst);
  UFE_CUDA(cudaGetLastError());
  UFE_CUDA(cudaStreamSynchronize(s));
  dev_free(tmp);
}

template <class T>
void to_external_t(ufe_ctx *ctx, T *h_dst, const T *d_src, bool tri, int ncols) {
  const int64_t n = tri ? ctx->nTri : ctx->nV;
  cudaStream_t s = ctx->stream;
  T *tmp = (T *)dev_alloc(sizeof(T) * n * ncols);
  k_gather_cols<T><<<blocks_for(n * ncols), 256, 0, s>>>(n, ncols, d_src, iperm_of(ctx, tri), tmp);
  UFE_CUDA(cudaGetLastError());
  UFE_CUDA(cudaMemcpyAsync(h_dst, tmp, sizeof(T) * n * ncols, cudaMemcpyDeviceToHost, s));
  UFE_CUDA(cudaStreamSynchronize(s));
  dev_free(tmp);
}

void to_internal(ufe_ctx *ctx, double *d_dst, const double *h_src, bool tri, int ncols) {
  to_internal_t<double>(ctx, d_dst, h_src, tri, ncols);
}
void to_internal_i32(ufe_ctx *ctx, int32_t *d_dst, const int32_t *h_src, bool tri) {
  to_internal_t<int32_t>(ctx, d_dst, h_src, tri, 1);
}
void to_external(ufe_ctx *ctx, double *h_dst, const double *d_src, bool tri, int ncols) {
  to_external_t<double>(ctx, h_dst, d_src, tri, ncols);
}

// Interleave two caller-ordered triangle fields into internal (u,v) pairs; a null field is 0.
void pair_to_internal(ufe_ctx *ctx, double2 *d_dst, const double *h_a, const double *h_b) {
  const int64_t n = ctx->nTri;
  cudaStream_t s = ctx->stream;
  double *ta = (double *)dev_alloc(sizeof(double) * n), *tb = (double *)dev_alloc(sizeof(double) * n);
  if (h_a) UFE_CUDA(cudaMemcpyAsync(ta, h_a, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  if (h_b) UFE_CUDA(cudaMemcpyAsync(tb, h_b, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  k_gather_pair<<<blocks_for(n), 256, 0, s>>>(n, h_a ? ta : nullptr, h_b ? tb : nullptr, ctx->perm_t, d_dst);
  UFE_CUDA(cudaGetLastError());
  UFE_CUDA(cudaStreamSynchronize(s));
  dev_free(ta);
  dev_free(tb);
}

void pair_to_external(ufe_ctx *ctx, double *h_a, double *h_b, const double2 *d_src) {
  const int64_t n = ctx->nTri;
  cudaStream_t s = ctx->stream;
  double *ta = (double *)dev_alloc(sizeof(double) * n), *tb = (double *)dev_alloc(sizeof(double) * n);
  k_scatter_pair<<<blocks_for(n), 256, 0, s>>>(n, d_src, ctx->iperm_t, ta, tb);
  UFE_CUDA(cudaGetLastError());
  if (h_a) UFE_CUDA(cudaMemcpyAsync(h_a, ta, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  if (h_b) UFE_CUDA(cudaMemcpyAsync(h_b, tb, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  UFE_CUDA(cudaStreamSynchronize(s));
  dev_free(ta);
  dev_free(tb);
}

// Row/column maps of an operator between internal and caller numbering.
static void op_maps(ufe_ctx *ctx, int op, const std::vector<int32_t> **row_perm, const std::vector<int32_t> **row_iperm,
                    const std::vector<int32_t> **col_perm, const std::vector<int32_t> **col_iperm) {
  const bool rows_tri = !(op == UFE_OP_MAP_B_A || op == UFE_OP_DDX_B_A || op == UFE_OP_DDY_B_A ||
                          op == UFE_OP_DDX_A_A || op == UFE_OP_DDY_A_A);
  const bool cols_tri = !(op == UFE_OP_MAP_A_B || op == UFE_OP_DDX_A_B || op == UFE_OP_DDY_A_B ||
                          op == UFE_OP_DDX_A_A || op == UFE_OP_DDY_A_A);
  *row_perm = rows_tri ? &ctx->perm_t_h : &ctx->perm_v_h;
  *row_iperm = rows_tri ? &ctx->iperm_t_h : &ctx->iperm_v_h;
  *col_perm = cols_tri ? &ctx->perm_t_h : &ctx->perm_v_h;
  *col_iperm = cols_tri ? &ctx->iperm_t_h : &ctx->iperm_v_h;
}

// caller CSR (0-based ptr/ind) -> internal CSR (rows reordered, columns renumbered, entry order kept)
void csr_to_internal(ufe_ctx *ctx, int op, const std::vector<int32_t> &ptr, const std::vector<int32_t> &ind,
                     const double *val, std::vector<int32_t> &iptr, std::vector<int32_t> &iind, std::vector<double> &ival) {
  const std::vector<int32_t> *rp, *rip, *cp, *cip;
  op_maps(ctx, op, &rp, &rip, &cp, &cip);
  const int64_t m = (int64_t)ptr.size() - 1;
  iptr.assign(m + 1, 0);
  iind.resize(ind.size());
  ival.resize(ind.size());
  for (int64_t i = 0; i < m; ++i) {
    int32_t r = (*rp)[i];
    iptr[i + 1] = iptr[i] + (ptr[r + 1] - ptr[r]);
  }
  for (int64_t i = 0; i < m; ++i) {
    int32_t r = (*rp)[i];
    int32_t q = iptr[i];
    for (int32_t k = ptr[r]; k < ptr[r + 1]; ++k, ++q) {
      iind[q] = (*cip)[ind[k]];
      ival[q] = val[k];
    }
  }
}

// internal CSR -> caller CSR (0-based)
void csr_to_external(ufe_ctx *ctx, int op, const std::vector<int32_t> &iptr, const std::vector<int32_t> &iind,
                     const std::vector<double> &ival, int32_t *ptr, int32_t *ind, double *val) {
  const std::vector<int32_t> *rp, *rip, *cp, *cip;
  op_maps(ctx, op, &rp, &rip, &cp, &cip);
  const int64_t m = (int64_t)iptr.size() - 1;
  std::vector<int32_t> p(m + 1, 0);
  for (int64_t r = 0; r < m; ++r) {
    int32_t i = (*rip)[r];
    p[r + 1] = p[r] + (iptr[i + 1] - iptr[i]);
  }
  if (ptr) std::copy(p.begin(), p.end(), ptr);
  for (int64_t r = 0; r < m; ++r) {
    int32_t i = (*rip)[r];
    int32_t q = p[r];
    for (int32_t k = iptr[i]; k < iptr[i + 1]; ++k, ++q) {
      if (ind) ind[q] = (*cp)[iind[k]];
      if (val) val[q] = ival[k];
    }
  }
}
