// Context, mesh upload, operators and CSR-algebra entry points of the C ABI.
#include <cstring>
#include <unordered_map>

#include "ufe_internal.cuh"

// ------------------------------------------------------------------------------------------
void *dev_alloc(size_t bytes) {
  void *p = nullptr;
  if (bytes == 0) bytes = 16;
  UFE_CUDA(cudaMalloc(&p, bytes));
  return p;
}

void dev_free(void *p) {
  if (p) cudaFree(p);
}

void free_operators(ufe_ctx *ctx) {
  for (void *p : ctx->op_allocs) dev_free(p);
  ctx->op_allocs.clear();
  for (int op = 0; op < UFE_OP_COUNT; ++op) {
    ctx->ops[op] = DevCSR{};
    ctx->op_set[op] = false;
  }
}

void ensure_reduce_area(ufe_ctx *ctx) {
  if (ctx->red.partials) return;
  ctx->red.partials = (double *)dev_alloc(sizeof(double) * kReduceSlots * kMaxReduceBlocks);
  ctx->red.tickets = (unsigned int *)dev_alloc(sizeof(unsigned int) * 64);
  UFE_CUDA(cudaMemsetAsync(ctx->red.tickets, 0, sizeof(unsigned int) * 64, ctx->stream));
}

int32_t pick_blocks(int64_t items, int threads, int max_blocks) {
  int64_t b = (items + threads - 1) / threads;
  if (b > max_blocks) b = max_blocks;
  if (b < 1) b = 1;
  return (int32_t)b;
}

static void free_mesh(ufe_ctx *ctx) {
  void *ptrs[] = {ctx->V, ctx->TriGC, ctx->zeta, ctx->nC, ctx->C, ctx->niTri, ctx->iTri,
                  ctx->VBI, ctx->Tri, ctx->TriC, ctx->TriBI};
  for (void *p : ptrs) dev_free(p);
  ctx->V = ctx->TriGC = ctx->zeta = nullptr;
  ctx->nC = ctx->C = ctx->niTri = ctx->iTri = ctx->VBI = ctx->Tri = ctx->TriC = ctx->TriBI = nullptr;
  free_layout(ctx);
  ctx->has_mesh = false;
}

template <class T>
static T *upload(const T *h, size_t n, cudaStream_t s) {
  T *d = (T *)dev_alloc(sizeof(T) * n);
  UFE_CUDA(cudaMemcpyAsync(d, h, sizeof(T) * n, cudaMemcpyHostToDevice, s));
  return d;
}

// ------------------------------------------------------------------------------------------
extern "C" void ufe_default_params(ufe_solver_params *p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  // defaults of model_configuration.f90:276-349,591-592
  p->choice_sliding_law = UFE_SLIDING_WEERTMAN;
  p->do_include_SSADIVA_crossterms = 1;
  p->do_GL_subgrid_friction = 1;
  p->BC_u_west = p->BC_u_east = p->BC_u_south = p->BC_u_north = UFE_BC_INFINITE;
  p->BC_v_west = p->BC_v_east = p->BC_v_south = p->BC_v_north = UFE_BC_INFINITE;
  p->visc_it_nit = 50;
  p->visc_it_norm_dUV_tol = 5e-5;
  p->visc_it_relax = 0.2;
  p->visc_eff_min = 1e4;
  p->vel_max = 5000.0;
  p->stress_balance_PETSc_rtol = 1e-7;
  p->stress_balance_PETSc_abstol = 1e-5;
  p->Glens_flow_law_exponent = 3.0;
  p->Glens_flow_law_epsilon_sq_0 = 1e-8;
  p->slid_Weertman_m = 3.0;
  p->slid_Budd_q_plastic = 0.3;
  p->slid_Budd_u_threshold = 100.0;
  p->subgrid_friction_exponent_on_B_grid = 2.0;
  p->slid_beta_max = 1e20;
  p->slid_delta_v = 1e-3;
  p->krylov_max_it = 10000;
  p->krylov_initial_guess = UFE_X0_CURRENT;
  p->precision = UFE_PREC_FP64;
  p->krylov_inner_rtol = 1e-2;
  p->krylov_forcing = 0.0;
  // model_configuration.f90:594-601
  p->choice_ice_rheology_Glen = UFE_RHEOLOGY_INPUT;
  p->choice_enhancement_factor_transition = UFE_ENH_SEPARATE;
  p->uniform_Glens_flow_factor = 1e-16;
  p->m_enh_sheet = 1.0;
  p->m_enh_shelf = 1.0;
  p->slid_ZI_p = 5.0;         // model_configuration.f90:336-337
  p->slid_ZI_ut = 200.0;
  p->SSA_icestream_Hi = 2000.0;   // the suggested values of :190-193
  p->SSA_icestream_dhdx = -0.0003;
  p->SSA_icestream_L = 150e3;
  p->SSA_icestream_m = 1.0;
}

extern "C" int32_t ufe_ctx_create(int32_t device, ufe_ctx **out) {
  if (!out) return UFE_ERR_INVALID;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) {
    cudaGetLastError();
    return UFE_ERR_DEVICE;
  }
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return UFE_ERR_DEVICE;
  // the kernels are built for sm_103a only
  if (!(prop.major == 10 && prop.minor == 3)) return UFE_ERR_DEVICE;
  ufe_ctx *ctx = new ufe_ctx();
  ctx->device = device;
  int32_t rc = guarded(ctx, [&]() -> int32_t {
    UFE_CUDA(cudaSetDevice(device));
    UFE_CUDA(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
    UFE_CUDA(cudaEventCreate(&ctx->ev0));
    UFE_CUDA(cudaEventCreate(&ctx->ev1));
    ensure_reduce_area(ctx);
    UFE_CUDA(cudaStreamSynchronize(ctx->stream));
    return UFE_OK;
  });
  if (rc != UFE_OK) {
    delete ctx;
    return rc;
  }
  *out = ctx;
  return UFE_OK;
}

extern "C" void ufe_ctx_destroy(ufe_ctx *ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  try {
    free_work(ctx);
  } catch (...) {
  }
  free_operators(ctx);
  free_mesh(ctx);
  dev_free(ctx->red.partials);
  dev_free(ctx->red.tickets);
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
}

extern "C" const char *ufe_ctx_last_error(const ufe_ctx *ctx) {
  return ctx ? ctx->last_error.c_str() : "null context";
}

extern "C" int32_t ufe_ctx_get_stream(ufe_ctx *ctx, void **stream) {
  return guarded(ctx, [&]() -> int32_t {
    UFE_REQUIRE(stream, UFE_ERR_INVALID, "null output");
    *stream = (void *)ctx->stream;
    return UFE_OK;
  });
}

extern "C" int32_t ufe_ctx_synchronize(ufe_ctx *ctx) {
  return guarded(ctx, [&]() -> int32_t {
    UFE_CUDA(cudaStreamSynchronize(ctx->stream));
    return UFE_OK;
  });
}

// ------------------------------------------------------------------------------------------
extern "C" int32_t ufe_mesh_upload(ufe_ctx *ctx, const ufe_mesh_desc *m) {
  return guarded(ctx, [&]() -> int32_t {
    UFE_REQUIRE(m, UFE_ERR_INVALID, "null mesh");
    UFE_REQUIRE(m->nV >= 3 && m->nTri >= 1 && m->nC_mem >= 3 && m->nz >= 2, UFE_ERR_INVALID,
                "mesh sizes out of range");
    UFE_REQUIRE(m->V && m->nC && m->C && m->niTri && m->iTri && m->VBI && m->Tri && m->TriC &&
                    m->TriBI && m->TriGC && m->zeta,
                UFE_ERR_INVALID, "mesh array missing");
    // index ranges (1-based, 0 = none where allowed); checked here so no kernel indexes out of bounds
    const int64_t nV = m->nV, nTri = m->nTri, nCm = m->nC_mem;
    for (int64_t t = 0; t < 3 * nTri; ++t) {
      UFE_REQUIRE(m->Tri[t] >= 1 && m->Tri[t] <= nV, UFE_ERR_INVALID, "Tri index out of range");
      UFE_REQUIRE(m->TriC[t] >= 0 && m->TriC[t] <= nTri, UFE_ERR_INVALID, "TriC index out of range");
    }
    for (int64_t v = 0; v < nV; ++v) {
      UFE_REQUIRE(m->nC[v] >= 1 && m->nC[v] <= nCm, UFE_ERR_INVALID, "nC out of range");
      UFE_REQUIRE(m->niTri[v] >= 1 && m->niTri[v] <= nCm, UFE_ERR_INVALID, "niTri out of range");
      for (int64_t c = 0; c < m->nC[v]; ++c) {
        int32_t j = m->C[c * nV + v];
        UFE_REQUIRE(j >= 1 && j <= nV, UFE_ERR_INVALID, "C index out of range");
      }
      for (int64_t c = 0; c < m->niTri[v]; ++c) {
        int32_t j = m->iTri[c * nV + v];
        UFE_REQUIRE(j >= 1 && j <= nTri, UFE_ERR_INVALID, "iTri index out of range");
      }
    }
    for (int64_t t = 0; t < nTri; ++t)
      UFE_REQUIRE(m->TriBI[t] >= 0 && m->TriBI[t] <= 8, UFE_ERR_INVALID, "TriBI out of range");
    UFE_CUDA(cudaSetDevice(ctx->device));
    UFE_CUDA(cudaStreamSynchronize(ctx->stream));
    free_work(ctx);
    free_operators(ctx);
    free_mesh(ctx);
    cudaStream_t s = ctx->stream;
    ctx->nV = m->nV;
    ctx->nTri = m->nTri;
    ctx->nC_mem = m->nC_mem;
    ctx->nz = m->nz;
    layout_upload_mesh(ctx, m);   // renumbered into the internal Z-order layout
    ctx->zeta = upload(m->zeta, m->nz, s);
    ctx->zeta_host.assign(m->zeta, m->zeta + m->nz);
    UFE_CUDA(cudaStreamSynchronize(s));
    ctx->has_mesh = true;
    return UFE_OK;
  });
}

extern "C" int32_t ufe_mesh_build_operators(ufe_ctx *ctx) {
  return guarded(ctx, [&]() -> int32_t {
    UFE_CUDA(cudaSetDevice(ctx->device));
    free_work(ctx);
    build_operators_gpu(ctx);
    return UFE_OK;
  });
}

static void expected_shape(ufe_ctx *ctx, int op, int32_t *m, int32_t *n) {
  switch (op) {
    case UFE_OP_MAP_A_B: case UFE_OP_DDX_A_B: case UFE_OP_DDY_A_B: *m = ctx->nTri; *n = ctx->nV; break;
    case UFE_OP_MAP_B_A: case UFE_OP_DDX_B_A: case UFE_OP_DDY_B_A: *m = ctx->nV; *n = ctx->nTri; break;
    case UFE_OP_DDX_A_A: case UFE_OP_DDY_A_A: *m = ctx->nV; *n = ctx->nV; break;
    default: *m = ctx->nTri; *n = ctx->nTri; break;
  }
}

static int family_first(int op) {
  if (op <= UFE_OP_DDY_A_B) return UFE_OP_MAP_A_B;
  if (op <= UFE_OP_DDY_B_A) return UFE_OP_MAP_B_A;
  if (op <= UFE_OP_DDY_A_A) return UFE_OP_DDX_A_A;
  return UFE_OP_M2_DDX_B_B;
}
static int family_last(int op) {
  if (op <= UFE_OP_DDY_A_B) return UFE_OP_DDY_A_B;
  if (op <= UFE_OP_DDY_B_A) return UFE_OP_DDY_B_A;
  if (op <= UFE_OP_DDY_A_A) return UFE_OP_DDY_A_A;
  return UFE_OP_M2_D2DY2_B_B;
}

extern "C" int32_t ufe_mesh_set_operator(ufe_ctx *ctx, int32_t op, int32_t m, int32_t n, int64_t nnz,
                                         const int32_t *ptr, const int32_t *ind, const double *val,
                                         int32_t index_base) {
  return guarded(ctx, [&]() -> int32_t {
    UFE_REQUIRE(ctx->has_mesh, UFE_ERR_INVALID, "no mesh uploaded");
    UFE_REQUIRE(op >= 0 && op < UFE_OP_COUNT, UFE_ERR_INVALID, "unknown operator");
    UFE_REQUIRE(index_base == 0 || index_base == 1, UFE_ERR_INVALID, "index_base must be 0 or 1");
    int32_t em, en;
    expected_shape(ctx, op, &em, &en);
    UFE_REQUIRE(m == em && n == en, UFE_ERR_INVALID, "operator shape does not match the mesh");
    UFE_REQUIRE(ptr && ind && val && nnz >= 0, UFE_ERR_INVALID, "null CSR array");
    std::vector<int32_t> hp(m + 1), hi((size_t)nnz);
    std::vector<double> val_int;
    for (int32_t i = 0; i <= m; ++i) hp[i] = ptr[i] - index_base;
    UFE_REQUIRE(hp[0] == 0 && hp[m] == nnz, UFE_ERR_INVALID, "CSR ptr does not span nnz");
    for (int32_t i = 0; i < m; ++i) UFE_REQUIRE(hp[i] <= hp[i + 1], UFE_ERR_INVALID, "CSR ptr not monotone");
    for (int64_t k = 0; k < nnz; ++k) {
      hi[k] = ind[k] - index_base;
      UFE_REQUIRE(hi[k] >= 0 && hi[k] < n, UFE_ERR_INVALID, "CSR column index out of range");
    }
    UFE_CUDA(cudaSetDevice(ctx->device));
    UFE_CUDA(cudaStreamSynchronize(ctx->stream));
    free_work(ctx);
    cudaStream_t s = ctx->stream;
    {
      std::vector<int32_t> ip, ii;
      std::vector<double> iv;
      csr_to_internal(ctx, op, hp, hi, val, ip, ii, iv);
      hp.swap(ip);
      hi.swap(ii);
      val_int.swap(iv);
    }
    DevCSR A;
    A.m = m; A.n = n; A.nnz = nnz;
    // share the pattern with a family member that has the same ptr/ind
    bool shared = false;
    for (int o = family_first(op); o <= family_last(op) && !shared; ++o) {
      if (o == op || !ctx->op_set[o] || ctx->ops[o].nnz != nnz) continue;
      std::vector<int32_t> op_ptr(m + 1), op_ind((size_t)nnz);
      UFE_CUDA(cudaMemcpy(op_ptr.data(), ctx->ops[o].ptr, sizeof(int32_t) * (m + 1), cudaMemcpyDeviceToHost));
      UFE_CUDA(cudaMemcpy(op_ind.data(), ctx->ops[o].ind, sizeof(int32_t) * nnz, cudaMemcpyDeviceToHost));
      if (op_ptr == hp && op_ind == hi) {
        A.ptr = ctx->ops[o].ptr;
        A.ind = ctx->ops[o].ind;
        shared = true;
      }
    }
    if (!shared) {
      A.ptr = upload(hp.data(), hp.size(), s);
      A.ind = upload(hi.data(), hi.size() ? hi.size() : 1, s);
      ctx->op_allocs.push_back(A.ptr);
      ctx->op_allocs.push_back(A.ind);
    }
    A.val = upload(val_int.data(), nnz ? (size_t)nnz : 1, s);
    ctx->op_allocs.push_back(A.val);
    UFE_CUDA(cudaStreamSynchronize(s));
    ctx->ops[op] = A;
    ctx->op_set[op] = true;
    return UFE_OK;
  });
}

extern "C" int32_t ufe_operator_info(ufe_ctx *ctx, int32_t op, int32_t *m, int32_t *n, int64_t *nnz) {
  return guarded(ctx, [&]() -> int32_t {
    UFE_REQUIRE(op >= 0 && op < UFE_OP_COUNT, UFE_ERR_INVALID, "unknown operator");
    UFE_REQUIRE(ctx->op_set[op], UFE_ERR_INVALID, "operator not built");
    if (m) *m = ctx->ops[op].m;
    if (n) *n = ctx->ops[op].n;
    if (nnz) *nnz = ctx->ops[op].nnz;
    return UFE_OK;
  });
}

extern "C" int32_t ufe_operator_export(ufe_ctx *ctx, int32_t op, int32_t *ptr, int32_t *ind, double *val,
                                       int32_t index_base) {
  return guarded(ctx, [&]() -> int32_t {
    UFE_REQUIRE(op >= 0 && op < UFE_OP_COUNT, UFE_ERR_INVALID, "unknown operator");
    UFE_REQUIRE(ctx->op_set[op], UFE_ERR_INVALID, "operator not built");
    UFE_REQUIRE(index_base == 0 || index_base == 1, UFE_ERR_INVALID, "index_base must be 0 or 1");
    const DevCSR &A = ctx->ops[op];
    UFE_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    std::vector<int32_t> ip(A.m + 1), ii(A.nnz);
    std::vector<double> iv(A.nnz);
    UFE_CUDA(cudaMemcpyAsync(ip.data(), A.ptr, sizeof(int32_t) * (A.m + 1), cudaMemcpyDeviceToHost, s));
    UFE_CUDA(cudaMemcpyAsync(ii.data(), A.ind, sizeof(int32_t) * A.nnz, cudaMemcpyDeviceToHost, s));
    UFE_CUDA(cudaMemcpyAsync(iv.data(), A.val, sizeof(double) * A.nnz, cudaMemcpyDeviceToHost, s));
    UFE_CUDA(cudaStreamSynchronize(s));
    csr_to_external(ctx, op, ip, ii, iv, ptr, ind, val);
    if (index_base) {
      if (ptr) for (int32_t i = 0; i <= A.m; ++i) ptr[i] += 1;
      if (ind) for (int64_t k = 0; k < A.nnz; ++k) ind[k] += 1;
    }
    return UFE_OK;
  });
}

extern "C" int32_t ufe_apply_operator(ufe_ctx *ctx, int32_t op, const double *x, double *y, int32_t ncols) {
  return guarded(ctx, [&]() -> int32_t {
    UFE_REQUIRE(op >= 0 && op < UFE_OP_COUNT, UFE_ERR_INVALID, "unknown operator");
    UFE_REQUIRE(ctx->op_set[op], UFE_ERR_INVALID, "operator not built");
    UFE_REQUIRE(x && y && ncols >= 1, UFE_ERR_INVALID, "bad vector arguments");
    const DevCSR &A = ctx->ops[op];
    UFE_CUDA(cudaSetDevice(ctx->device));
    cudaStream_t s = ctx->stream;
    const bool rows_tri = !(op == UFE_OP_MAP_B_A || op == UFE_OP_DDX_B_A || op == UFE_OP_DDY_B_A ||
                            op == UFE_OP_DDX_A_A || op == UFE_OP_DDY_A_A);
    const bool cols_tri = !(op == UFE_OP_MAP_A_B || op == UFE_OP_DDX_A_B || op == UFE_OP_DDY_A_B ||
                            op == UFE_OP_DDX_A_A || op == UFE_OP_DDY_A_A);
    double *dx = (double *)dev_alloc(sizeof(double) * (size_t)A.n * ncols);
    double *dy = (double *)dev_alloc(sizeof(double) * (size_t)A.m * ncols);
    to_internal(ctx, dx, x, cols_tri, ncols);
    launch_csr_spmv(s, A, dx, dy, ncols);
    to_external(ctx, y, dy, rows_tri, ncols);
    dev_free(dx);
    dev_free(dy);
    return UFE_OK;
  });
}

// Validate and upload a caller CSR matrix as a 0-based device matrix.
static DevCSR upload_csr(ufe_ctx *ctx, int32_t m, int32_t n, int64_t nnz, const int32_t *ptr,
                         const int32_t *ind, const double *val, int32_t index_base,
                         std::vector<void *> &owned) {
  UFE_REQUIRE(m >= 1 && n >= 1 && nnz >= 0, UFE_ERR_INVALID, "bad matrix sizes");
  UFE_REQUIRE(ptr && ind && val, UFE_ERR_INVALID, "null CSR array");
  UFE_REQUIRE(index_base == 0 || index_base == 1, UFE_ERR_INVALID, "index_base must be 0 or 1");
  std::vector<int32_t> hp(m + 1), hi((size_t)nnz);
  for (int32_t i = 0; i <= m; ++i) hp[i] = ptr[i] - index_base;
  UFE_REQUIRE(hp[0] == 0 && hp[m] == nnz, UFE_ERR_INVALID, "CSR ptr does not span nnz");
  for (int32_t i = 0; i < m; ++i) UFE_REQUIRE(hp[i] <= hp[i + 1], UFE_ERR_INVALID, "CSR ptr not monotone");
  for (int64_t k = 0; k < nnz; ++k) {
    hi[k] = ind[k] - index_base;
    UFE_REQUIRE(hi[k] >= 0 && hi[k] < n, UFE_ERR_INVALID, "CSR column index out of range");
  }
  cudaStream_t s = ctx->stream;
  DevCSR A;
  A.m = m; A.n = n; A.nnz = nnz;
  A.ptr = upload(hp.data(), hp.size(), s);
  A.ind = upload(hi.data(), hi.size() ? hi.size() : 1, s);
  A.val = upload(val, nnz ? (size_t)nnz : 1, s);
  owned.push_back(A.ptr);
  owned.push_back(A.ind);
  owned.push_back(A.val);
  return A;
}

extern "C" int32_t ufe_csr_spmv(ufe_ctx *ctx, int32_t m, int32_t n, int64_t nnz, const int32_t *ptr,
                                const int32_t *ind, const double *val, int32_t index_base,
                                const double *x, double *y, int32_t ncols) {
  std::vector<void *> owned;
  int32_t rc = guarded(ctx, [&]() -> int32_t {
    UFE_REQUIRE(x && y && ncols >= 1, UFE_ERR_INVALID, "bad vector arguments");
    UFE_CUDA(cudaSetDevice(ctx->device));
    DevCSR A = upload_csr(ctx, m, n, nnz, ptr, ind, val, index_base, owned);
    cudaStream_t s = ctx->stream;
    double *dx = upload(x, (size_t)n * ncols, s);
    owned.push_back(dx);
    double *dy = (double *)dev_alloc(sizeof(double) * (size_t)m * ncols);
    owned.push_back(dy);
    launch_csr_spmv(s, A, dx, dy, ncols);
    UFE_CUDA(cudaMemcpyAsync(y, dy, sizeof(double) * (size_t)m * ncols, cudaMemcpyDeviceToHost, s));
    UFE_CUDA(cudaStreamSynchronize(s));
    return UFE_OK;
  });
  if (ctx) cudaStreamSynchronize(ctx->stream);
  for (void *p : owned) dev_free(p);
  return rc;
}

extern "C" int32_t ufe_solve_csr(ufe_ctx *ctx, int32_t m, int64_t nnz, const int32_t *ptr,
                                 const int32_t *ind, const double *val, int32_t index_base,
                                 const double *bb, double *xx, double rtol, double abstol,
                                 int32_t max_it, int32_t *n_Axb_its) {
  std::vector<void *> owned;
  int32_t rc = guarded(ctx, [&]() -> int32_t {
    UFE_REQUIRE(bb && xx, UFE_ERR_INVALID, "bad vector arguments");
    UFE_REQUIRE(max_it >= 1 && rtol >= 0.0 && abstol >= 0.0, UFE_ERR_INVALID, "bad tolerances");
    UFE_CUDA(cudaSetDevice(ctx->device));
    DevCSR A = upload_csr(ctx, m, m, nnz, ptr, ind, val, index_base, owned);
    cudaStream_t s = ctx->stream;
    double *db = upload(bb, (size_t)m, s);
    owned.push_back(db);
    double *dx = upload(xx, (size_t)m, s);
    owned.push_back(dx);
    int32_t its = 0;
    int32_t st = solve_csr_device(ctx, A, db, dx, rtol, abstol, max_it, &its);
    UFE_CUDA(cudaMemcpyAsync(xx, dx, sizeof(double) * m, cudaMemcpyDeviceToHost, s));
    UFE_CUDA(cudaStreamSynchronize(s));
    if (n_Axb_its) *n_Axb_its = its;
    return st;
  });
  if (ctx) cudaStreamSynchronize(ctx->stream);
  for (void *p : owned) dev_free(p);
  return rc;
}
