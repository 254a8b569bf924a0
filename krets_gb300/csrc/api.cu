// C ABI (include/krets_gpu.h): handle management, program upload, workspace layout,
// launches, CUDA-graph replay of the plain transient, timing and error reporting.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "kernels.cuh"
#include "warp_kernels.cuh"
#include "adjoint.cuh"
#include "krets_gpu.h"
#include "symbolic.h"

using namespace krets;

namespace {

thread_local std::string g_last_error;
std::atomic<long long> g_launches{0};

krets_status fail(krets_status s, const std::string &msg) {
  g_last_error = msg;
  return s;
}

#define CU(call)                                                                         \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess)                                                               \
      return fail(KRETS_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

struct LayBuilder {
  Lay L{};
  size_t cur = 0;
  int idx = 0;
  void add(int slot, size_t bytes) {
    L.off[slot] = (int)cur;
    cur = align16(cur + bytes);
  }
  Lay done() {
    L.bytes = align16(cur ? cur : 16);
    return L;
  }
};

// Uploaded program: one device buffer holding every index array.
struct DevProgram {
  Program host;
  DevProg view{};
  void *buf = nullptr;
  ~DevProgram() { if (buf) cudaFree(buf); }
};

int device_sm_count() {
  static int sms = -1;
  if (sms < 0) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      sms = 1;
  }
  return sms;
}

size_t max_smem_optin() {
  static int v = -1;
  if (v < 0) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
      v = 48 * 1024;
  }
  return (size_t)v;
}

bool is_device_ptr(const void *p) {
  if (!p) return false;
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

}  // namespace

struct krets_circuit {
  std::vector<krets_element> el;
  int n = 0, ne = 0;
  KCfg cfg{};
  bool nonlinear = false;
  krets_element *d_el = nullptr;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[4] = {};
  float kernel_ms = 0.f, call_ms = 0.f;
  std::map<std::string, std::unique_ptr<DevProgram>> progs;
  int *d_is_cur_tmp = nullptr;
  // scratch
  void *scratch = nullptr;
  size_t scratch_bytes = 0;
  int *d_small = nullptr;  // counters / status words
  unsigned long long *d_hist = nullptr;
  long long hist[8] = {};
  int fallbacks = 0;
  int warps_per_cta = 0, grid = 0;
  void *l2buf = nullptr;

  ~krets_circuit() {
    if (d_el) cudaFree(d_el);
    if (scratch) cudaFree(scratch);
    if (d_small) cudaFree(d_small);
    if (d_hist) cudaFree(d_hist);
    if (l2buf) cudaFree(l2buf);
    for (auto &e : ev)
      if (e) cudaEventDestroy(e);
    if (stream) cudaStreamDestroy(stream);
  }

  krets_status ensure_scratch(size_t bytes) {
    if (bytes <= scratch_bytes) return KRETS_OK;
    if (scratch) cudaFree(scratch);
    scratch = nullptr;
    scratch_bytes = 0;
    CU(cudaMalloc(&scratch, bytes));
    scratch_bytes = bytes;
    return KRETS_OK;
  }
};

namespace {

krets_status upload_program(krets_circuit *c, Program &&P, DevProgram &D) {
  D.host = std::move(P);
  Program &H = D.host;
  // compute lu_src: A entry index per LU slot
  std::vector<int> lu_src(H.lu_col.size(), -1);
  for (size_t t = 0; t < H.a_slot.size(); ++t) lu_src[H.a_slot[t]] = (int)t;
  std::vector<int> is_cur(H.n, 0);
  for (int e = 0; e < H.ne; ++e)
    if (H.el_pos[4 * e + 2] >= 0) is_cur[H.el_pos[4 * e + 2]] = 1;
  struct Part { const void *src; size_t bytes; size_t off; };
  std::vector<Part> parts;
  size_t total = 0;
  auto add = [&](const void *src, size_t bytes) {
    parts.push_back({src, bytes, total});
    total = align16(total + (bytes ? bytes : 4));
    return parts.size() - 1;
  };
  auto vi = [&](const std::vector<int> &v) { return add(v.data(), v.size() * sizeof(int)); };
  size_t i_q = vi(H.q), i_rp = vi(H.lu_rowptr), i_col = vi(H.lu_col), i_dg = vi(H.lu_diag), i_src = vi(lu_src);
  size_t i_arp = vi(H.a_rowptr), i_acol = vi(H.a_col), i_acp = vi(H.a_cptr), i_acn = vi(H.a_contrib);
  size_t i_bcp = vi(H.b_cptr), i_bcn = vi(H.b_contrib), i_pp = vi(H.piv_ptr), i_pv = vi(H.piv), i_up = vi(H.upd);
  size_t i_lp = vi(H.lev_ptr), i_lr = vi(H.lev_rows), i_ulp = vi(H.ulev_ptr), i_ulr = vi(H.ulev_rows);
  size_t i_ep = vi(H.el_pos), i_ic = vi(is_cur);
  size_t i_qi = vi(H.qinv), i_ld = vi(H.ldesc), i_ud = vi(H.udesc), i_rp2 = vi(H.res_ptr), i_ro = vi(H.res_op);
  size_t i_dy = vi(H.dyn_e), i_bdp = vi(H.bd_ptr), i_bdo = vi(H.bd_op), i_sp = vi(H.sprog);
  size_t i_tp = vi(H.tprog), i_pr = vi(H.prow);
  CU(cudaMalloc(&D.buf, total));
  std::vector<char> staging(total, 0);
  for (auto &p : parts)
    if (p.bytes) memcpy(staging.data() + p.off, p.src, p.bytes);
  CU(cudaMemcpy(D.buf, staging.data(), total, cudaMemcpyHostToDevice));
  char *b = (char *)D.buf;
  auto ptr = [&](size_t i) { return (const void *)(b + parts[i].off); };
  DevProg &V = D.view;
  V.n = H.n;
  V.ne = H.ne;
  V.nnz_a = (int)H.a_col.size();
  V.nnz_lu = (int)H.lu_col.size();
  V.nlev = (int)H.lev_ptr.size() - 1;
  V.nulev = (int)H.ulev_ptr.size() - 1;
  V.mode = H.mode;
  V.method = H.method;
  V.q = (const int *)ptr(i_q);
  V.lu_rowptr = (const int *)ptr(i_rp);
  V.lu_col = (const int *)ptr(i_col);
  V.lu_diag = (const int *)ptr(i_dg);
  V.lu_src = (const int *)ptr(i_src);
  V.a_rowptr = (const int *)ptr(i_arp);
  V.a_col = (const int *)ptr(i_acol);
  V.a_cptr = (const int *)ptr(i_acp);
  V.a_contrib = (const int *)ptr(i_acn);
  V.b_cptr = (const int *)ptr(i_bcp);
  V.b_contrib = (const int *)ptr(i_bcn);
  V.piv_ptr = (const int *)ptr(i_pp);
  V.piv = (const int4 *)ptr(i_pv);
  V.upd = (const int2 *)ptr(i_up);
  V.lev_ptr = (const int *)ptr(i_lp);
  V.lev_rows = (const int *)ptr(i_lr);
  V.ulev_ptr = (const int *)ptr(i_ulp);
  V.ulev_rows = (const int *)ptr(i_ulr);
  V.el_pos = (const int4 *)ptr(i_ep);
  V.is_cur = (const int *)ptr(i_ic);
  V.el = c->d_el;
  V.qinv = (const int *)ptr(i_qi);
  V.ldesc = (const int4 *)ptr(i_ld);
  V.udesc = (const int4 *)ptr(i_ud);
  V.res_ptr = (const int *)ptr(i_rp2);
  V.res_op = (const int2 *)ptr(i_ro);
  V.dyn_e = (const int *)ptr(i_dy);
  V.bd_ptr = (const int *)ptr(i_bdp);
  V.bd_op = (const int *)ptr(i_bdo);
  V.ndyn = (int)H.dyn_e.size();
  V.ncap = H.ncap;
  V.n_resop = (int)H.res_op.size() / 2;
  V.sprog = (const int *)ptr(i_sp);
  for (int k = 0; k < 14; ++k) V.sp_off[k] = H.sp_off[k];
  V.sprog_ok = H.sprog_ok;
  V.tprog = (const int *)ptr(i_tp);
  for (int k = 0; k < 8; ++k) V.tp_off[k] = H.tp_off[k];
  V.n_utlev = H.n_utlev;
  V.n_ltlev = H.n_ltlev;
  V.prow = (const int *)ptr(i_pr);
  bool nl = false;
  for (int e = 0; e < H.ne; ++e) {
    int k = c->el[e].kind;
    if (H.mode == MODE_DC && k == KRETS_ELEM_C) continue;
    if (k == KRETS_ELEM_D || k == KRETS_ELEM_M || k == KRETS_ELEM_Q) nl = true;
  }
  V.nonlinear = nl;
  return KRETS_OK;
}

krets_status get_program(krets_circuit *c, int mode, int method, double h, double f, DevProgram **out) {
  char key[128];
  snprintf(key, sizeof key, "%d/%d/%.17g/%.17g", mode, method, mode == MODE_TRAN ? h : 0.0, mode == MODE_AC ? f : 0.0);
  auto it = c->progs.find(key);
  if (it != c->progs.end()) {
    *out = it->second.get();
    return KRETS_OK;
  }
  Program P;
  std::string msg;
  int st = build_program(c->el.data(), c->ne, c->n, mode, method, h, f, -1, P, msg);
  if (st != KRETS_OK) return fail(st, msg);
  auto D = std::make_unique<DevProgram>();
  krets_status s2 = upload_program(c, std::move(P), *D);
  if (s2 != KRETS_OK) return s2;
  *out = D.get();
  c->progs[key] = std::move(D);
  return KRETS_OK;
}

Lay layout_op(const DevProg &P) {
  LayBuilder B;
  B.add(0, sizeof(double) * P.nnz_lu);
  B.add(1, sizeof(double) * P.n);
  B.add(2, sizeof(double) * P.n);
  B.add(3, sizeof(double) * P.n);
  B.add(4, sizeof(double) * P.ne);
  B.add(5, sizeof(double) * P.ne);
  B.add(6, sizeof(int) * 4);
  B.add(7, sizeof(double) * P.ne);
  return B.done();
}

Lay layout_tran(const DevProg &P, bool mixed) {
  LayBuilder B;
  B.add(0, sizeof(double) * P.ne);
  B.add(1, mixed ? sizeof(double) * P.nnz_a : 0);
  B.add(2, (mixed ? sizeof(float) : sizeof(double)) * P.nnz_lu);
  B.add(3, sizeof(double) * P.n);
  B.add(4, P.nonlinear ? sizeof(double) * P.n : 0);
  B.add(5, P.nonlinear ? sizeof(double) * P.n : 0);
  B.add(6, sizeof(double) * P.n);
  B.add(7, mixed ? sizeof(float) * P.n : 0);
  B.add(8, sizeof(double) * P.ne);
  B.add(9, sizeof(double) * P.ne);
  B.add(10, sizeof(double) * P.ne);
  B.add(11, sizeof(double) * 32);
  B.add(12, sizeof(int) * 4);
  B.add(13, sizeof(int) * 4);
  return B.done();
}

Lay layout_ac(const DevProg &P, bool mixed) {
  LayBuilder B;
  B.add(0, sizeof(double) * P.ne);
  B.add(1, mixed ? 16 * (size_t)P.nnz_a : 0);
  B.add(2, (mixed ? 8 : 16) * (size_t)P.nnz_lu);
  B.add(3, 16 * (size_t)P.n);
  B.add(4, 16 * (size_t)P.n);
  B.add(5, mixed ? 8 * (size_t)P.n : 0);
  B.add(6, sizeof(double) * P.ne);
  B.add(7, sizeof(double) * P.ne);
  B.add(8, sizeof(double) * P.ne);
  B.add(9, sizeof(double) * P.n);
  B.add(10, sizeof(double) * 32);
  B.add(11, sizeof(int) * 4);
  B.add(12, sizeof(int) * 4);
  return B.done();
}

// Decide shared vs global placement and the grid for a per-CTA workspace.
template <typename K>
krets_status plan_launch(krets_circuit *c, K kernel, const Lay &L, int threads, int items, int &grid,
                         size_t &smem, char *&gws) {
  if (L.bytes <= max_smem_optin()) {
    smem = L.bytes;
    gws = nullptr;
    CU(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem));
    if (per_sm < 1) per_sm = 1;
    grid = std::max(1, std::min(items, per_sm * device_sm_count()));
  } else {
    smem = 0;
    grid = std::max(1, std::min(items, 2 * device_sm_count()));
    krets_status s = c->ensure_scratch(L.bytes * (size_t)grid);
    if (s != KRETS_OK) return s;
    gws = (char *)c->scratch;
  }
  return KRETS_OK;
}

krets_status map_status(int bits, int mode_for_decomp) {
  if (bits & KS_NOTIMPL) return fail(KRETS_ERR_NOT_IMPLEMENTED, "stamp is not implemented in the reference (todo!())");
  if (bits & (KS_SINGULAR | KS_NONFINITE))
    return fail(mode_for_decomp == 0 ? KRETS_ERR_MATRIX_DECOMPOSITION : KRETS_ERR_DECOMPOSITION_FAILED,
                "zero or non-finite pivot during factorisation");
  if (bits & KS_MAXITER) return fail(KRETS_ERR_MAX_ITERATIONS, "maximum Newton iterations exceeded");
  if (bits & KS_STALL) return fail(KRETS_ERR_PIVOT_UNSTABLE, "iterative refinement stalled");
  return KRETS_OK;
}

struct DevBuf {
  void *p = nullptr;
  ~DevBuf() { if (p) cudaFree(p); }
};

// Device view of a caller buffer: use it directly when it is device memory, otherwise a
// temporary device buffer (copied in when `in` is set).
krets_status dev_view(const void *user, size_t bytes, bool in, cudaStream_t s, DevBuf &tmp, void **dptr) {
  if (!user || bytes == 0) {
    *dptr = nullptr;
    return KRETS_OK;
  }
  if (is_device_ptr(user)) {
    *dptr = const_cast<void *>(user);
    return KRETS_OK;
  }
  CU(cudaMalloc(&tmp.p, bytes));
  if (in) CU(cudaMemcpyAsync(tmp.p, user, bytes, cudaMemcpyHostToDevice, s));
  *dptr = tmp.p;
  return KRETS_OK;
}

krets_status run_op(krets_circuit *c, DevProgram *D, int n_inst, const double *d_values, double *d_x,
                    size_t out_stride, int *d_status, int *d_iters, int threads) {
  Lay L = layout_op(D->view);
  int grid;
  size_t smem;
  char *gws;
  krets_status s = plan_launch(c, k_op, L, threads, n_inst, grid, smem, gws);
  if (s != KRETS_OK) return s;
  k_op<<<grid, threads, smem, c->stream>>>(D->view, c->cfg, L, gws, d_values, d_x, out_stride, d_status, d_iters,
                                          n_inst);
  g_launches++;
  CU(cudaGetLastError());
  return KRETS_OK;
}

int plain_threads(const DevProg &P) {
  int t = 128;
  while (t < 512 && t < P.n / 2) t *= 2;
  return t;
}

}  // namespace

// ============================================ fixed scratch for the allocation-free entry
// krets_batch_tran_noalloc() keeps all of its scratch (work-queue counter, refinement
// statistics, per-instance operating-point status, FP64 fallback factors) in this array
// instead of allocating it.  It is 16 MiB, lives on every GPU that loads the library until
// the process exits, and is shared by every call on that GPU.
#define KRETS_NOALLOC_SCRATCH_BYTES (16u << 20)
static __device__ __align__(256) unsigned char g_noalloc_scratch[KRETS_NOALLOC_SCRATCH_BYTES];

namespace {

// Device address of g_noalloc_scratch per device, looked up once per device (the host-side
// name of the array is only a stand-in, never a device address).
constexpr int kMaxDevices = 64;
void *g_noalloc_addr[kMaxDevices] = {};

krets_status noalloc_scratch_address(void **out) {
  int dev = 0;
  CU(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return fail(KRETS_ERR_CUDA, "device index out of range");
  if (!g_noalloc_addr[dev]) {
    void *p = nullptr;
    CU(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    g_noalloc_addr[dev] = p;
  }
  *out = g_noalloc_addr[dev];
  return KRETS_OK;
}

// Lookup without building: the allocation-free entry uses only programs that an earlier
// call already compiled and uploaded.
DevProgram *find_program(krets_circuit *c, int mode, int method, double h, double f) {
  char key[128];
  snprintf(key, sizeof key, "%d/%d/%.17g/%.17g", mode, method, mode == MODE_TRAN ? h : 0.0, mode == MODE_AC ? f : 0.0);
  auto it = c->progs.find(key);
  return it == c->progs.end() ? nullptr : it->second.get();
}

// OR of the operating-point and transient statuses, folded into the caller's per-instance
// status array, plus one summary word.
__global__ void k_status_fold(const int *op_status, int *inst_status, int n, int *any) {
  int acc = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int v = op_status[i] | inst_status[i];
    inst_status[i] = v;
    acc |= v;
  }
  if (acc) atomicOr(any, acc);
}

}  // namespace

// ====================================================================== C ABI
extern "C" {

krets_status krets_circuit_create(const krets_element *elems, int32_t n_elem, int32_t n_unknowns,
                                  const krets_config *cfg, krets_circuit **out) {
  if (!out || (!elems && n_elem > 0) || n_elem < 0 || n_unknowns <= 0)
    return fail(KRETS_ERR_INVALID_ARGUMENT, "invalid arguments to krets_circuit_create");
  *out = nullptr;
  for (int e = 0; e < n_elem; ++e) {
    const krets_element &x = elems[e];
    if (x.kind < KRETS_ELEM_R || x.kind > KRETS_ELEM_Q)
      return fail(KRETS_ERR_INVALID_ELEMENT, "unknown element kind at index " + std::to_string(e));
    const int idx[4] = {x.p, x.m, x.b, x.g};
    for (int v : idx)
      if (v < -1 || v >= n_unknowns)
        return fail(KRETS_ERR_INVALID_ARGUMENT, "element " + std::to_string(e) + " has an unknown index out of range");
  }
  int dev_count = 0;
  if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count == 0) {
    cudaGetLastError();
    return fail(KRETS_ERR_CUDA, "no CUDA device is available (this library has no CPU fallback)");
  }
  auto c = std::make_unique<krets_circuit>();
  c->el.assign(elems, elems + n_elem);
  c->n = n_unknowns;
  c->ne = n_elem;
  krets_config d{0.001, 1e-12, 1e-6, 300, 0};
  const krets_config &k = cfg ? *cfg : d;
  c->cfg = KCfg{k.relative_tolerance, k.current_absolute_tolerance, k.voltage_absolute_tolerance,
                k.maximum_iterations};
  CU(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  for (auto &e : c->ev) CU(cudaEventCreate(&e));
  CU(cudaMalloc(&c->d_el, sizeof(krets_element) * std::max(1, n_elem)));
  if (n_elem) CU(cudaMemcpy(c->d_el, elems, sizeof(krets_element) * n_elem, cudaMemcpyHostToDevice));
  CU(cudaMalloc(&c->d_small, 4096));
  CU(cudaMalloc(&c->d_hist, 8 * sizeof(unsigned long long)));
  *out = c.release();
  return KRETS_OK;
}

krets_status krets_circuit_destroy(krets_circuit *c) {
  delete c;
  return KRETS_OK;
}

krets_status krets_circuit_info(const krets_circuit *cc, int32_t mode, int32_t *n, int32_t *nnz_a, int32_t *nnz_lu,
                                int32_t *n_levels, int32_t *n_ulevels) {
  krets_circuit *c = const_cast<krets_circuit *>(cc);
  if (!c) return fail(KRETS_ERR_INVALID_ARGUMENT, "null circuit");
  DevProgram *D;
  krets_status s = get_program(c, mode, KRETS_METHOD_TR, 1e-12, 1e3, &D);
  if (s != KRETS_OK) return s;
  if (n) *n = D->view.n;
  if (nnz_a) *nnz_a = D->view.nnz_a;
  if (nnz_lu) *nnz_lu = D->view.nnz_lu;
  if (n_levels) *n_levels = D->view.nlev;
  if (n_ulevels) *n_ulevels = D->view.nulev;
  return KRETS_OK;
}

krets_status krets_op(krets_circuit *c, double *x_out, int32_t *iters_out) {
  if (!c || !x_out) return fail(KRETS_ERR_INVALID_ARGUMENT, "null argument");
  DevProgram *D;
  krets_status s = get_program(c, MODE_DC, 0, 0, 0, &D);
  if (s != KRETS_OK) return s == KRETS_ERR_DECOMPOSITION_FAILED ? KRETS_ERR_MATRIX_DECOMPOSITION : s;
  DevBuf tx;
  void *dx;
  CU(cudaEventRecord(c->ev[0], c->stream));
  s = dev_view(x_out, sizeof(double) * c->n, false, c->stream, tx, &dx);
  if (s) return s;
  int *d_status = c->d_small, *d_iters = c->d_small + 1;
  CU(cudaMemsetAsync(c->d_small, 0, 16, c->stream));
  CU(cudaEventRecord(c->ev[2], c->stream));
  s = run_op(c, D, 1, nullptr, (double *)dx, c->n, d_status, d_iters, plain_threads(D->view));
  if (s) return s;
  CU(cudaEventRecord(c->ev[3], c->stream));
  if (tx.p) CU(cudaMemcpyAsync(x_out, dx, sizeof(double) * c->n, cudaMemcpyDeviceToHost, c->stream));
  int h[2];
  CU(cudaMemcpyAsync(h, c->d_small, sizeof h, cudaMemcpyDeviceToHost, c->stream));
  CU(cudaEventRecord(c->ev[1], c->stream));
  CU(cudaStreamSynchronize(c->stream));
  cudaEventElapsedTime(&c->kernel_ms, c->ev[2], c->ev[3]);
  cudaEventElapsedTime(&c->call_ms, c->ev[0], c->ev[1]);
  if (iters_out) *iters_out = h[1];
  return map_status(h[0], 0);
}

krets_status krets_batch_op(krets_circuit *c, int32_t n_inst, const double *values, double *x_out,
                            int32_t *inst_status) {
  if (!c || !x_out || n_inst <= 0) return fail(KRETS_ERR_INVALID_ARGUMENT, "invalid arguments");
  DevProgram *D;
  krets_status s = get_program(c, MODE_DC, 0, 0, 0, &D);
  if (s != KRETS_OK) return s;
  CU(cudaEventRecord(c->ev[0], c->stream));
  DevBuf tv, tx, ts;
  void *dv, *dx, *dst;
  s = dev_view(values, sizeof(double) * c->ne * (size_t)n_inst, true, c->stream, tv, &dv);
  if (s) return s;
  s = dev_view(x_out, sizeof(double) * c->n * (size_t)n_inst, false, c->stream, tx, &dx);
  if (s) return s;
  CU(cudaMalloc(&ts.p, sizeof(int) * n_inst));
  dst = ts.p;
  CU(cudaMemsetAsync(dst, 0, sizeof(int) * n_inst, c->stream));
  CU(cudaEventRecord(c->ev[2], c->stream));
  s = run_op(c, D, n_inst, (const double *)dv, (double *)dx, c->n, (int *)dst, nullptr, 128);
  if (s) return s;
  CU(cudaEventRecord(c->ev[3], c->stream));
  if (tx.p) CU(cudaMemcpyAsync(x_out, dx, sizeof(double) * c->n * (size_t)n_inst, cudaMemcpyDeviceToHost, c->stream));
  std::vector<int> st(n_inst);
  CU(cudaMemcpyAsync(st.data(), dst, sizeof(int) * n_inst, cudaMemcpyDeviceToHost, c->stream));
  CU(cudaEventRecord(c->ev[1], c->stream));
  CU(cudaStreamSynchronize(c->stream));
  cudaEventElapsedTime(&c->kernel_ms, c->ev[2], c->ev[3]);
  cudaEventElapsedTime(&c->call_ms, c->ev[0], c->ev[1]);
  int any = 0;
  for (int i = 0; i < n_inst; ++i) {
    if (inst_status) inst_status[i] = st[i];
    any |= st[i];
  }
  return map_status(any, 0);
}

krets_status krets_dc(krets_circuit *c, int32_t sweep_elem, double start, double stop, double step, double *x_out,
                      int32_t max_points, int32_t *n_points) {
  if (!c || !x_out) return fail(KRETS_ERR_INVALID_ARGUMENT, "null argument");
  if (sweep_elem < 0 || sweep_elem >= c->ne) return fail(KRETS_ERR_ELEMENT_NOT_FOUND, "sweep element not found");
  int kind = c->el[sweep_elem].kind;
  if (kind != KRETS_ELEM_V && kind != KRETS_ELEM_I)
    return fail(KRETS_ERR_INVALID_ELEMENT, "DC sweep element must be a voltage or current source");
  double np_d = std::fabs((stop - start) / step);
  if (!(np_d < 1e9)) return fail(KRETS_ERR_INVALID_ARGUMENT, "invalid sweep range");
  int np = (int)np_d + 1;  // dc.rs:153-154 (truncation)
  if (n_points) *n_points = np;
  if (np > max_points) return fail(KRETS_ERR_INVALID_ARGUMENT, "x_out too small for the sweep");
  DevProgram *D;
  krets_status s = get_program(c, MODE_DC, 0, 0, 0, &D);
  if (s != KRETS_OK) return s;
  CU(cudaEventRecord(c->ev[0], c->stream));
  DevBuf tx;
  void *dx;
  s = dev_view(x_out, sizeof(double) * c->n * (size_t)np, false, c->stream, tx, &dx);
  if (s) return s;
  Lay L = layout_op(D->view);
  int threads = plain_threads(D->view), grid;
  size_t smem;
  char *gws;
  s = plan_launch(c, k_dc_sweep, L, threads, 1, grid, smem, gws);
  if (s) return s;
  CU(cudaEventRecord(c->ev[2], c->stream));
  k_dc_sweep<<<1, threads, smem, c->stream>>>(D->view, c->cfg, L, gws, sweep_elem, start, step, np, (double *)dx,
                                              c->d_small);
  g_launches++;
  CU(cudaGetLastError());
  CU(cudaEventRecord(c->ev[3], c->stream));
  if (tx.p) CU(cudaMemcpyAsync(x_out, dx, sizeof(double) * c->n * (size_t)np, cudaMemcpyDeviceToHost, c->stream));
  int h = 0;
  CU(cudaMemcpyAsync(&h, c->d_small, sizeof h, cudaMemcpyDeviceToHost, c->stream));
  CU(cudaEventRecord(c->ev[1], c->stream));
  CU(cudaStreamSynchronize(c->stream));
  cudaEventElapsedTime(&c->kernel_ms, c->ev[2], c->ev[3]);
  cudaEventElapsedTime(&c->call_ms, c->ev[0], c->ev[1]);
  return map_status(h, 1);
}

krets_status krets_batch_ac(krets_circuit *c, int32_t n_inst, const double *values, const double *freqs,
                            int32_t n_freq, int32_t precision, double *x_out, int32_t *item_status) {
  if (!c || !freqs || !x_out || n_inst <= 0 || n_freq <= 0) return fail(KRETS_ERR_INVALID_ARGUMENT, "invalid arguments");
  std::vector<double> hf(n_freq);
  if (is_device_ptr(freqs)) CU(cudaMemcpy(hf.data(), freqs, sizeof(double) * n_freq, cudaMemcpyDeviceToHost));
  else memcpy(hf.data(), freqs, sizeof(double) * n_freq);
  double lo = 1e300, hi = 0;
  for (double f : hf) {
    if (!(f > 0)) return fail(KRETS_ERR_INVALID_ARGUMENT, "batched AC frequencies must be > 0");
    lo = std::min(lo, f);
    hi = std::max(hi, f);
  }
  DevProgram *Ddc, *Dac;
  krets_status s = get_program(c, MODE_DC, 0, 0, 0, &Ddc);
  if (s != KRETS_OK) return s;
  double frep = std::sqrt(lo * hi);
  s = get_program(c, MODE_AC, 0, 0, frep, &Dac);
  if (s != KRETS_OK) return s;
  CU(cudaEventRecord(c->ev[0], c->stream));
  DevBuf tv, tf, tx, top, ts;
  void *dv, *df, *dx;
  s = dev_view(values, sizeof(double) * c->ne * (size_t)n_inst, true, c->stream, tv, &dv);
  if (s) return s;
  s = dev_view(freqs, sizeof(double) * n_freq, true, c->stream, tf, &df);
  if (s) return s;
  size_t out_bytes = sizeof(double) * 2 * c->n * (size_t)n_freq * n_inst;
  s = dev_view(x_out, out_bytes, false, c->stream, tx, &dx);
  if (s) return s;
  CU(cudaMalloc(&top.p, sizeof(double) * c->n * (size_t)n_inst));
  size_t items = (size_t)n_inst * n_freq;
  CU(cudaMalloc(&ts.p, sizeof(int) * (items + n_inst)));
  int *d_item_st = (int *)ts.p, *d_op_st = d_item_st + items;
  CU(cudaMemsetAsync(ts.p, 0, sizeof(int) * (items + n_inst), c->stream));
  s = run_op(c, Ddc, n_inst, (const double *)dv, (double *)top.p, c->n, d_op_st, nullptr, 128);
  if (s) return s;
  bool mixed = precision == KRETS_PREC_MIXED;
  Lay L = layout_ac(Dac->view, mixed);
  int threads = 128, grid;
  size_t smem;
  char *gws;
  auto kern = mixed ? k_ac_batch<1> : k_ac_batch<0>;
  s = plan_launch(c, kern, L, threads, (int)std::min<size_t>(items, 1 << 30), grid, smem, gws);
  if (s) return s;
  int *queue = c->d_small + 8;
  CU(cudaMemsetAsync(queue, 0, sizeof(int), c->stream));
  CU(cudaEventRecord(c->ev[2], c->stream));
  kern<<<grid, threads, smem, c->stream>>>(Dac->view, L, gws, (const double *)dv, (const double *)top.p, n_inst,
                                           (const double *)df, n_freq, (double *)dx, d_item_st, queue);
  g_launches++;
  CU(cudaGetLastError());
  CU(cudaEventRecord(c->ev[3], c->stream));
  if (tx.p) CU(cudaMemcpyAsync(x_out, dx, out_bytes, cudaMemcpyDeviceToHost, c->stream));
  std::vector<int> st(items + n_inst);
  CU(cudaMemcpyAsync(st.data(), d_item_st, sizeof(int) * (items + n_inst), cudaMemcpyDeviceToHost, c->stream));
  CU(cudaEventRecord(c->ev[1], c->stream));
  CU(cudaStreamSynchronize(c->stream));
  cudaEventElapsedTime(&c->kernel_ms, c->ev[2], c->ev[3]);
  cudaEventElapsedTime(&c->call_ms, c->ev[0], c->ev[1]);
  int any_op = 0, any = 0;
  for (size_t i = 0; i < items; ++i) {
    if (item_status) item_status[i] = st[i];
    any |= st[i];
  }
  for (int i = 0; i < n_inst; ++i) any_op |= st[items + i];
  if (any_op) return map_status(any_op, 0);
  return map_status(any, 1);
}

krets_status krets_ac(krets_circuit *c, const double *freqs, int32_t n_freq, double *x_out, int32_t *n_kept) {
  if (!c || (!freqs && n_freq > 0) || !x_out) return fail(KRETS_ERR_INVALID_ARGUMENT, "null argument");
  std::vector<double> kept;
  for (int i = 0; i < n_freq; ++i)
    if (freqs[i] > 0.0) kept.push_back(freqs[i]);  // ac.rs:40-45
  if (n_kept) *n_kept = (int)kept.size();
  if (kept.empty()) {
    // the reference still computes the operating point first (ac.rs:25)
    std::vector<double> xop(c->n);
    return krets_op(c, xop.data(), nullptr);
  }
  return krets_batch_ac(c, 1, nullptr, kept.data(), (int)kept.size(), KRETS_PREC_FP64, x_out, nullptr);
}

krets_status krets_tran(krets_circuit *c, double h, int32_t n_steps, int32_t method, int32_t source_lag,
                        int32_t refactor_each_step, double *x_out) {
  if (!c || !x_out || n_steps < 0 || !(h > 0)) return fail(KRETS_ERR_INVALID_ARGUMENT, "invalid arguments");
  DevProgram *Ddc, *Dtr;
  krets_status s = get_program(c, MODE_DC, 0, 0, 0, &Ddc);
  if (s != KRETS_OK) return s;
  s = get_program(c, MODE_TRAN, method, h, 0, &Dtr);
  if (s != KRETS_OK) return s;
  CU(cudaEventRecord(c->ev[0], c->stream));
  size_t out_bytes = sizeof(double) * c->n * ((size_t)n_steps + 1);
  DevBuf tx, stbuf;
  void *dx;
  s = dev_view(x_out, out_bytes, false, c->stream, tx, &dx);
  if (s) return s;
  const DevProg &P = Dtr->view;
  size_t nd = 8 * (size_t)P.n + 3 * (size_t)P.ne + P.nnz_lu + 64;
  CU(cudaMalloc(&stbuf.p, nd * sizeof(double)));
  CU(cudaMemsetAsync(stbuf.p, 0, nd * sizeof(double), c->stream));
  double *d = (double *)stbuf.p;
  TranState st;
  st.x = d; d += P.n;
  st.prev = d; d += P.n;
  st.guess = d; d += P.n;
  st.b = d; d += P.n;
  st.ca = d; d += P.ne;
  st.cb = d; d += P.ne;
  st.icap = d; d += P.ne;
  st.lu = d; d += P.nnz_lu;
  int *ints = (int *)d;
  st.status = ints;
  st.step = ints + 2;
  st.factored = ints + 4;
  int *op_status = ints + 6;
  CU(cudaEventRecord(c->ev[2], c->stream));
  s = run_op(c, Ddc, 1, nullptr, (double *)dx, c->n, op_status, nullptr, plain_threads(Ddc->view));
  if (s) return s;
  // TRAN state starts from the operating point (position space of the TRAN program)
  k_gather<<<(P.n + 255) / 256, 256, 0, c->stream>>>(st.x, (const double *)dx, P.q, P.n);
  g_launches++;
  int threads = plain_threads(P);
  if (n_steps > 0) {
    // a CUDA graph of up to 256 step launches, replayed; each launch advances one step
    int chunk = std::min(n_steps, 256);
    cudaGraph_t graph;
    cudaGraphExec_t exec;
    CU(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    for (int i = 0; i < chunk; ++i)
      k_tran_step<<<1, threads, 0, c->stream>>>(P, c->cfg, st, h, method, source_lag, refactor_each_step, n_steps,
                                               (double *)dx);
    CU(cudaStreamEndCapture(c->stream, &graph));
    CU(cudaGraphInstantiate(&exec, graph, 0));
    int reps = (n_steps + chunk - 1) / chunk;
    for (int r = 0; r < reps; ++r) CU(cudaGraphLaunch(exec, c->stream));
    g_launches += (long long)reps * chunk;
    CU(cudaStreamSynchronize(c->stream));
    cudaGraphExecDestroy(exec);
    cudaGraphDestroy(graph);
  }
  CU(cudaEventRecord(c->ev[3], c->stream));
  if (tx.p) CU(cudaMemcpyAsync(x_out, dx, out_bytes, cudaMemcpyDeviceToHost, c->stream));
  int h2[8];
  CU(cudaMemcpyAsync(h2, ints, sizeof h2, cudaMemcpyDeviceToHost, c->stream));
  CU(cudaEventRecord(c->ev[1], c->stream));
  CU(cudaStreamSynchronize(c->stream));
  cudaEventElapsedTime(&c->kernel_ms, c->ev[2], c->ev[3]);
  cudaEventElapsedTime(&c->call_ms, c->ev[0], c->ev[1]);
  if (h2[6]) return map_status(h2[6], 0);
  return map_status(h2[0], 1);
}

krets_status krets_batch_tran(krets_circuit *c, int32_t n_inst, const double *values, double h, int32_t n_steps,
                              int32_t method, int32_t source_lag, int32_t precision, double *x_out,
                              int32_t *inst_status) {
  if (!c || !x_out || n_inst <= 0 || n_steps < 0 || !(h > 0)) return fail(KRETS_ERR_INVALID_ARGUMENT, "invalid arguments");
  DevProgram *Ddc, *Dtr;
  krets_status s = get_program(c, MODE_DC, 0, 0, 0, &Ddc);
  if (s != KRETS_OK) return s;
  s = get_program(c, MODE_TRAN, method, h, 0, &Dtr);
  if (s != KRETS_OK) return s;
  CU(cudaEventRecord(c->ev[0], c->stream));
  size_t stride = (size_t)c->n * ((size_t)n_steps + 1);
  DevBuf tv, tx, ts, tfb;
  void *dv, *dx;
  s = dev_view(values, sizeof(double) * c->ne * (size_t)n_inst, true, c->stream, tv, &dv);
  if (s) return s;
  s = dev_view(x_out, sizeof(double) * stride * n_inst, false, c->stream, tx, &dx);
  if (s) return s;
  CU(cudaMalloc(&ts.p, sizeof(int) * 2 * (size_t)n_inst));
  int *d_st = (int *)ts.p, *d_opst = d_st + n_inst;
  CU(cudaMemsetAsync(ts.p, 0, sizeof(int) * 2 * (size_t)n_inst, c->stream));
  s = run_op(c, Ddc, n_inst, (const double *)dv, (double *)dx, stride, d_opst, nullptr, 128);
  if (s) return s;
  const bool dfd = precision == KRETS_PREC_DF;
  bool mixed = precision == KRETS_PREC_MIXED;
  const DevProg &P = Dtr->view;
  if (dfd && P.nonlinear) mixed = true;  // nonlinear circuits: refactor per Newton iteration (FP32 + refinement)
  int *queue = c->d_small + 8;
  int *d_fallbacks = c->d_small + 12;
  CU(cudaMemsetAsync(c->d_small + 8, 0, 8 * sizeof(int), c->stream));
  CU(cudaMemsetAsync(c->d_hist, 0, 8 * sizeof(unsigned long long), c->stream));
  const char *eng = getenv("KRETS_ENGINE");
  bool warp_engine = !(eng && strcmp(eng, "block") == 0);
  WarpLay WL{};
  size_t per_warp = 0;
  if (warp_engine) {
    size_t cur = 0;
    auto put = [&](int &off, size_t bytes) { off = (int)cur; cur = align16(cur + bytes); };
    put(WL.lu, (mixed ? 4 : 8) * (size_t)P.nnz_lu);
    put(WL.coef, 8 * (size_t)P.ne);
    put(WL.x, 8 * (size_t)P.n);
    put(WL.b, 8 * (size_t)P.n);
    put(WL.w, mixed ? 4 * (size_t)P.n : 16);  // double-float direct: the group's 4 status words
    put(WL.cb, 8 * (size_t)P.ndyn);
    put(WL.icap, 8 * (size_t)P.ncap);
    put(WL.prev, P.nonlinear ? 8 * (size_t)P.n : 0);
    put(WL.guess, P.nonlinear ? 8 * (size_t)P.n : 0);
    WL.bytes = (int)align16(cur);
    WL.sprog_bytes = (int)align16((size_t)P.sp_off[11] * sizeof(int));
    per_warp = WL.bytes;
    if (!P.sprog_ok || per_warp + WL.sprog_bytes > max_smem_optin()) warp_engine = false;
  }
  double *fb = nullptr;
  // double-float direct: one instance per group of G threads (default 128); it stages only
  // the step-program words before the residual operators, so it fits where the warp
  // engine may not
  DfdLay DL{};
  bool use_dfd = dfd && !P.nonlinear && P.sprog_ok && !(eng && strcmp(eng, "block") == 0);
  if (use_dfd) {
    size_t cur = 0;
    auto put = [&](int &off, size_t bytes) { off = (int)cur; cur = align16(cur + bytes); };
    put(DL.lu, 8 * (size_t)P.nnz_lu);
    put(DL.x, 8 * (size_t)P.n);
    put(DL.cdyn, 8 * (size_t)P.ndyn);
    put(DL.cb, 8 * (size_t)P.ndyn);
    put(DL.icap, 8 * (size_t)P.ncap);
    DL.coef64 = DL.x;  // set-up scratch over x / cdyn / cb / icap (+ padding if needed)
    if (cur - DL.x < 8 * (size_t)P.ne) cur = DL.x + align16(8 * (size_t)P.ne);
    put(DL.slot, 16);
    DL.bytes = (int)align16(cur);
    DL.sprog_bytes = (int)align16((size_t)P.sp_off[5] * sizeof(int));
    if ((size_t)DL.bytes + DL.sprog_bytes > max_smem_optin()) use_dfd = false;
  }
  if (use_dfd) {
    const char *genv = getenv("KRETS_GROUP");
    int G = genv ? atoi(genv) : 128;
    if (G != 32 && G != 64 && G != 128) G = 128;
    int W = (int)std::max<size_t>(1, std::min<size_t>(640 / G, (max_smem_optin() - DL.sprog_bytes) / DL.bytes));
    const size_t smem = DL.sprog_bytes + (size_t)W * DL.bytes;
    const char *oenv = getenv("KRETS_DFD_OPTS");
    const int opts = oenv ? atoi(oenv) : 0;
    void (*kd)(DevProg, KCfg, DfdLay, const double *, int, double, int, int, int, double *, int *, int *, int) =
        G == 32 ? k_tran_dfd<32> : (G == 64 ? k_tran_dfd<64> : k_tran_dfd<128>);
    CU(cudaFuncSetAttribute(kd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kd, G * W, smem));
    if (per_sm < 1) return fail(KRETS_ERR_CUDA, "double-float engine does not fit on an SM");
    int grid = std::max(1, std::min((n_inst + W - 1) / W, per_sm * device_sm_count()));
    c->warps_per_cta = W * G / 32;
    c->grid = grid;
    CU(cudaEventRecord(c->ev[2], c->stream));
    kd<<<grid, G * W, smem, c->stream>>>(P, c->cfg, DL, (const double *)dv, n_inst, h, n_steps, method, source_lag,
                                        (double *)dx, d_st, queue, opts);
  } else if (warp_engine) {
    const char *bud = getenv("KRETS_SMEM_BUDGET");
    size_t budget = bud ? (size_t)atol(bud) : max_smem_optin();
    budget = std::min(budget, max_smem_optin());
    int W = (int)std::max<size_t>(1, std::min<size_t>(8, (budget - WL.sprog_bytes) / per_warp));
    const char *wenv = getenv("KRETS_WARPS_PER_CTA");
    if (wenv) W = std::max(1, std::min(8, atoi(wenv)));
    while (W > 1 && WL.sprog_bytes + (size_t)W * per_warp > max_smem_optin()) --W;
    size_t smem = WL.sprog_bytes + (size_t)W * per_warp;
    auto kern = mixed ? k_tran_warp<1> : k_tran_warp<0>;
    // linear circuits in mixed precision take the double-float variant (FP32 pipes)
    const char *dfenv = getenv("KRETS_DF");
    const bool use_df = mixed && !P.nonlinear && !(dfenv && dfenv[0] == '0');
    CU(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    CU(cudaFuncSetAttribute(k_tran_warp_df, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    if (use_df) CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tran_warp_df, 32 * W, smem));
    else CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32 * W, smem));
    if (per_sm < 1) return fail(KRETS_ERR_CUDA, "warp engine does not fit on an SM");
    int grid = std::max(1, std::min((n_inst + W - 1) / W, per_sm * device_sm_count()));
    if (mixed) {
      CU(cudaMalloc(&tfb.p, sizeof(double) * (size_t)P.nnz_lu * grid * W));
      fb = (double *)tfb.p;
    }
    const char *tenv = getenv("KRETS_REFINE_TOL");
    double tol = tenv ? atof(tenv) : 1e-8;
    c->warps_per_cta = W;
    c->grid = grid;
    CU(cudaEventRecord(c->ev[2], c->stream));
    if (use_df)
      k_tran_warp_df<<<grid, 32 * W, smem, c->stream>>>(P, c->cfg, WL, (const double *)dv, n_inst, h, n_steps, method,
                                                       source_lag, (double *)dx, d_st, queue, c->d_hist, (float)tol);
    else
      kern<<<grid, 32 * W, smem, c->stream>>>(P, c->cfg, WL, (const double *)dv, n_inst, h, n_steps, method,
                                             source_lag, (double *)dx, d_st, queue, c->d_hist, d_fallbacks, fb, tol);
  } else {
    Lay L = layout_tran(P, mixed);
    int threads = 128, grid;
    size_t smem;
    char *gws;
    auto kern = mixed ? k_tran_batch<1> : k_tran_batch<0>;
    s = plan_launch(c, kern, L, threads, n_inst, grid, smem, gws);
    if (s) return s;
    if (mixed) {
      CU(cudaMalloc(&tfb.p, sizeof(double) * (size_t)P.nnz_lu * grid));
      fb = (double *)tfb.p;
    }
    c->warps_per_cta = 0;
    c->grid = grid;
    CU(cudaEventRecord(c->ev[2], c->stream));
    kern<<<grid, threads, smem, c->stream>>>(P, c->cfg, L, gws, (const double *)dv, n_inst, h, n_steps, method,
                                             source_lag, (double *)dx, d_st, queue, c->d_hist, d_fallbacks, fb);
  }
  g_launches++;
  CU(cudaGetLastError());
  CU(cudaEventRecord(c->ev[3], c->stream));
  if (tx.p) CU(cudaMemcpyAsync(x_out, dx, sizeof(double) * stride * n_inst, cudaMemcpyDeviceToHost, c->stream));
  std::vector<int> st(2 * (size_t)n_inst);
  CU(cudaMemcpyAsync(st.data(), ts.p, sizeof(int) * 2 * (size_t)n_inst, cudaMemcpyDeviceToHost, c->stream));
  unsigned long long hist[8];
  CU(cudaMemcpyAsync(hist, c->d_hist, sizeof hist, cudaMemcpyDeviceToHost, c->stream));
  int fbk = 0;
  CU(cudaMemcpyAsync(&fbk, d_fallbacks, sizeof fbk, cudaMemcpyDeviceToHost, c->stream));
  CU(cudaEventRecord(c->ev[1], c->stream));
  CU(cudaStreamSynchronize(c->stream));
  cudaEventElapsedTime(&c->kernel_ms, c->ev[2], c->ev[3]);
  cudaEventElapsedTime(&c->call_ms, c->ev[0], c->ev[1]);
  for (int k = 0; k < 8; ++k) c->hist[k] = (long long)hist[k];
  c->fallbacks = fbk;
  int any = 0, any_op = 0;
  for (int i = 0; i < n_inst; ++i) {
    int v = st[i] | st[n_inst + i];
    if (inst_status) inst_status[i] = v;
    any |= st[i];
    any_op |= st[n_inst + i];
  }
  if (any_op) return map_status(any_op, 0);
  return map_status(any, 1);
}

krets_status krets_adjoint_tran(krets_circuit *c, int32_t n_inst, const double *values, double h, int32_t n_steps,
                                int32_t method, int32_t out_unknown, int32_t checkpoint_every, int32_t gradient,
                                double *loss_out, double *grad_out) {
  if (!c || n_inst <= 0 || n_steps <= 0 || !(h > 0) || !loss_out || (gradient && !grad_out) || checkpoint_every <= 0 ||
      out_unknown < 0 || out_unknown >= c->n)
    return fail(KRETS_ERR_INVALID_ARGUMENT, "invalid arguments to krets_adjoint_tran");
  DevProgram *Ddc, *Dtr;
  krets_status s = get_program(c, MODE_DC, 0, 0, 0, &Ddc);
  if (s != KRETS_OK) return s;
  s = get_program(c, MODE_TRAN, method, h, 0, &Dtr);
  if (s != KRETS_OK) return s;
  const DevProg &P = Dtr->view;
  const Program &H = Dtr->host;
  if (P.nonlinear) return fail(KRETS_ERR_NOT_IMPLEMENTED, "adjoint sensitivities need a linear circuit");
  if (!P.sprog_ok) return fail(KRETS_ERR_INVALID_ARGUMENT, "circuit too large for the adjoint engine");
  CU(cudaEventRecord(c->ev[0], c->stream));
  DevBuf tv, top, tbufs, tck, tseg, tloss, tgrad, tst;
  void *dv;
  s = dev_view(values, sizeof(double) * c->ne * (size_t)n_inst, true, c->stream, tv, &dv);
  if (s) return s;
  // the recurrence starts from x_0 = 0: check that the operating point is zero
  CU(cudaMalloc(&top.p, sizeof(double) * c->n * (size_t)n_inst + sizeof(int) * (size_t)n_inst));
  int *op_st = (int *)((double *)top.p + (size_t)c->n * n_inst);
  s = run_op(c, Ddc, n_inst, (const double *)dv, (double *)top.p, c->n, op_st, nullptr, 128);
  if (s) return s;
  std::vector<double> opx((size_t)c->n * n_inst);
  CU(cudaMemcpyAsync(opx.data(), top.p, sizeof(double) * opx.size(), cudaMemcpyDeviceToHost, c->stream));
  CU(cudaStreamSynchronize(c->stream));
  for (double v : opx)
    if (v != 0.0)
      return fail(KRETS_ERR_NOT_IMPLEMENTED, "adjoint sensitivities need a zero operating point at t = 0 "
                                             "(sources at 0 when the transient starts)");
  // per-element adjoint descriptors and the column map of C^T lambda
  std::vector<int> adj(4 * (size_t)P.ne, -1), ccp(P.n + 1, 0), cco;
  std::vector<std::vector<int>> cols(P.n);
  for (int e = 0; e < P.ne; ++e) {
    const krets_element &E = c->el[e];
    if ((E.kind == KRETS_ELEM_R || E.kind == KRETS_ELEM_C) && (E.flags & KRETS_FLAG_G2))
      return fail(KRETS_ERR_NOT_IMPLEMENTED, "adjoint sensitivities of group-2 resistor/capacitor stamps");
    adj[4 * e] = E.kind;
    adj[4 * e + 1] = E.p >= 0 ? H.pinv[E.p] : -1;
    adj[4 * e + 2] = E.m >= 0 ? H.pinv[E.m] : -1;
    adj[4 * e + 3] = E.b >= 0 ? H.pinv[E.b] : -1;
  }
  for (size_t d = 0; d < H.dyn_e.size(); ++d) {
    const krets_element &E = c->el[H.dyn_e[d]];
    if (E.kind == KRETS_ELEM_C) {
      if (E.p >= 0) cols[H.qinv[E.p]].push_back((int)d << 1);
      if (E.m >= 0) cols[H.qinv[E.m]].push_back(((int)d << 1) | 1);
    } else if (E.kind == KRETS_ELEM_L && E.b >= 0) {
      cols[H.qinv[E.b]].push_back((int)d << 1);
    }
  }
  for (int k = 0; k < P.n; ++k) {
    cco.insert(cco.end(), cols[k].begin(), cols[k].end());
    ccp[k + 1] = (int)cco.size();
  }
  size_t nb = sizeof(int) * (adj.size() + ccp.size() + cco.size() + 8);
  CU(cudaMalloc(&tbufs.p, nb));
  int *d_adj = (int *)tbufs.p, *d_ccp = d_adj + adj.size(), *d_cco = d_ccp + ccp.size();
  CU(cudaMemcpyAsync(d_adj, adj.data(), sizeof(int) * adj.size(), cudaMemcpyHostToDevice, c->stream));
  CU(cudaMemcpyAsync(d_ccp, ccp.data(), sizeof(int) * ccp.size(), cudaMemcpyHostToDevice, c->stream));
  if (!cco.empty()) CU(cudaMemcpyAsync(d_cco, cco.data(), sizeof(int) * cco.size(), cudaMemcpyHostToDevice, c->stream));
  // shared-memory layout: step program, transposed program, then one slice per instance
  // shared memory: step program, transposed program, then the instance's arrays
  AdjLay AL{};
  size_t cur = 0;
  auto put = [&](int &off, size_t bytes) { off = (int)cur; cur = align16(cur + bytes); };
  put(AL.slot, 16);
  put(AL.lu, 8 * (size_t)P.nnz_lu);
  put(AL.x, 8 * (size_t)P.n);
  put(AL.cdyn, 8 * (size_t)P.ndyn);
  put(AL.cb, 8 * (size_t)P.ndyn);
  put(AL.icap, 8 * (size_t)P.ncap);
  put(AL.lam, 8 * (size_t)P.n);
  put(AL.cba, 8 * (size_t)P.ndyn);
  AL.coef64 = AL.x;  // set-up scratch over x .. cba (dead once the LU is formed)
  if (cur - AL.x < 8 * (size_t)P.ne) cur = AL.x + align16(8 * (size_t)P.ne);
  AL.bytes = (int)align16(cur);
  AL.sprog_bytes = (int)align16((size_t)P.sp_off[5] * sizeof(int));
  AL.tprog_bytes = (int)align16((size_t)P.tp_off[5] * sizeof(int));
  const size_t smem = (size_t)AL.sprog_bytes + AL.tprog_bytes + AL.bytes;
  if (smem > max_smem_optin())
    return fail(KRETS_ERR_INVALID_ARGUMENT, "circuit too large for the adjoint engine's shared memory");
  // per-thread register caches: n <= 4 x 256, ndyn <= 4 x 256, ne <= 8 x 256
  constexpr int RK = 4, RD = 4, RE = 8;
  if (P.n > RK * kAdjHalf || P.ndyn > RD * kAdjHalf || P.ne > RE * kAdjHalf)
    return fail(KRETS_ERR_INVALID_ARGUMENT,
                "circuit too large for the adjoint engine (n > 1024, more than 1024 C/L/V/I or ne > 2048)");
  auto ka = k_adjoint_dfd<RK, RD, RE>;
  CU(cudaFuncSetAttribute(ka, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ka, kAdjThreads, smem));
  if (per_sm < 1) return fail(KRETS_ERR_CUDA, "adjoint engine does not fit on an SM");
  const int grid = std::max(1, std::min(n_inst, per_sm * device_sm_count()));
  const int K = std::min(checkpoint_every, n_steps);
  const int J = (n_steps + K - 1) / K;
  CU(cudaMalloc(&tck.p, sizeof(df) * (size_t)grid * J * ((size_t)P.n + P.ncap)));
  // three segment buffers of K+1 states and two lambda histories of K vectors per CTA
  const size_t seg_bytes = sizeof(df) * (size_t)grid * 3 * ((size_t)K + 1) * P.n;
  const size_t hist_bytes = sizeof(df) * (size_t)grid * 2 * (size_t)K * P.n;
  CU(cudaMalloc(&tseg.p, gradient ? seg_bytes + hist_bytes : 16));
  df *d_hist = gradient ? (df *)((char *)tseg.p + seg_bytes) : nullptr;
  DevBuf dl_loss, dl_grad;
  void *d_loss, *d_grad = nullptr;
  s = dev_view(loss_out, sizeof(double) * n_inst, false, c->stream, dl_loss, &d_loss);
  if (s) return s;
  if (gradient) {
    s = dev_view(grad_out, sizeof(double) * (size_t)n_inst * c->ne, false, c->stream, dl_grad, &d_grad);
    if (s) return s;
  }
  CU(cudaMalloc(&tst.p, sizeof(int) * n_inst));
  CU(cudaMemsetAsync(tst.p, 0, sizeof(int) * n_inst, c->stream));
  int *queue = c->d_small + 8;
  CU(cudaMemsetAsync(queue, 0, sizeof(int), c->stream));
  CU(cudaEventRecord(c->ev[2], c->stream));
  ka<<<grid, kAdjThreads, smem, c->stream>>>(P, AL, (const double *)dv, n_inst, h, n_steps, method, K,
                                             H.qinv[out_unknown], (const int4 *)d_adj, d_ccp, d_cco, (df *)tck.p,
                                             (df *)tseg.p, d_hist, (double *)d_loss, (double *)d_grad, (int *)tst.p,
                                             queue, gradient ? 1 : 0);
  g_launches++;
  CU(cudaGetLastError());
  CU(cudaEventRecord(c->ev[3], c->stream));
  if (dl_loss.p) CU(cudaMemcpyAsync(loss_out, d_loss, sizeof(double) * n_inst, cudaMemcpyDeviceToHost, c->stream));
  if (dl_grad.p)
    CU(cudaMemcpyAsync(grad_out, d_grad, sizeof(double) * (size_t)n_inst * c->ne, cudaMemcpyDeviceToHost, c->stream));
  std::vector<int> st(n_inst);
  CU(cudaMemcpyAsync(st.data(), tst.p, sizeof(int) * n_inst, cudaMemcpyDeviceToHost, c->stream));
  CU(cudaEventRecord(c->ev[1], c->stream));
  CU(cudaStreamSynchronize(c->stream));
  cudaEventElapsedTime(&c->kernel_ms, c->ev[2], c->ev[3]);
  cudaEventElapsedTime(&c->call_ms, c->ev[0], c->ev[1]);
  c->warps_per_cta = kAdjThreads / 32;
  c->grid = grid;
  int any = 0;
  for (int v : st) any |= v;
  return map_status(any, 1);
}

const char *krets_status_string(krets_status s) {
  switch (s) {
    case KRETS_OK: return "ok";
    case KRETS_ERR_ELEMENT_NOT_FOUND: return "element not found in the netlist";
    case KRETS_ERR_MAX_ITERATIONS: return "maximum iterations exceeded";
    case KRETS_ERR_INVALID_ELEMENT: return "invalid element format";
    case KRETS_ERR_UNEXPECTED: return "unexpected error";
    case KRETS_ERR_DECOMPOSITION_FAILED: return "decomposition failed";
    case KRETS_ERR_MATRIX_BUILD: return "matrix build failed";
    case KRETS_ERR_MATRIX_DECOMPOSITION: return "matrix decomposition failed";
    case KRETS_ERR_NOT_IMPLEMENTED: return "not implemented in the reference";
    case KRETS_ERR_TIMEOUT: return "device wait timed out";
    case KRETS_ERR_CUDA: return "CUDA error";
    case KRETS_ERR_INVALID_ARGUMENT: return "invalid argument";
    case KRETS_ERR_OUT_OF_MEMORY: return "out of memory";
    case KRETS_ERR_PIVOT_UNSTABLE: return "pivot unstable / refinement stalled";
  }
  return "unknown status";
}

const char *krets_last_error_message(void) { return g_last_error.c_str(); }

krets_status krets_last_timing(const krets_circuit *c, float *kernel_ms, float *call_ms) {
  if (!c) return fail(KRETS_ERR_INVALID_ARGUMENT, "null circuit");
  if (kernel_ms) *kernel_ms = c->kernel_ms;
  if (call_ms) *call_ms = c->call_ms;
  return KRETS_OK;
}

int64_t krets_launch_count(void) { return g_launches.load(); }

krets_status krets_last_refine_stats(const krets_circuit *c, int64_t histogram[8], int32_t *fallbacks) {
  if (!c) return fail(KRETS_ERR_INVALID_ARGUMENT, "null circuit");
  if (histogram)
    for (int k = 0; k < 8; ++k) histogram[k] = c->hist[k];
  if (fallbacks) *fallbacks = c->fallbacks;
  return KRETS_OK;
}

krets_status krets_device_alloc(size_t bytes, void **ptr) {
  if (!ptr) return fail(KRETS_ERR_INVALID_ARGUMENT, "null pointer");
  cudaError_t e = cudaMalloc(ptr, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(e == cudaErrorMemoryAllocation ? KRETS_ERR_OUT_OF_MEMORY : KRETS_ERR_CUDA, cudaGetErrorString(e));
  }
  return KRETS_OK;
}

krets_status krets_device_free(void *ptr) {
  CU(cudaFree(ptr));
  return KRETS_OK;
}

krets_status krets_memcpy_h2d(void *dst, const void *src, size_t bytes) {
  CU(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice));
  return KRETS_OK;
}

krets_status krets_memcpy_d2h(void *dst, const void *src, size_t bytes) {
  CU(cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost));
  return KRETS_OK;
}

krets_status krets_flush_l2(krets_circuit *c) {
  if (!c) return fail(KRETS_ERR_INVALID_ARGUMENT, "null circuit");
  const size_t n = (size_t)64 << 20;  // 512 MB of doubles, several times the L2
  if (!c->l2buf) CU(cudaMalloc(&c->l2buf, n * sizeof(double)));
  k_fill<<<4 * device_sm_count(), 256, 0, c->stream>>>((double *)c->l2buf, n, 1.0);
  CU(cudaGetLastError());
  CU(cudaStreamSynchronize(c->stream));
  return KRETS_OK;
}

krets_status krets_device_synchronize(void) {
  CU(cudaDeviceSynchronize());
  return KRETS_OK;
}

// Batched transient for callers that must not allocate device memory (see krets_gpu.h).
// Same kernels and results as krets_batch_tran with device-resident buffers; the scratch
// that call would allocate comes from g_noalloc_scratch.
krets_status krets_batch_tran_noalloc(krets_circuit *c, int32_t n_inst, const double *d_values, double h,
                                      int32_t n_steps, int32_t method, int32_t source_lag, int32_t precision,
                                      double *d_x_out, int32_t *d_inst_status) {
  if (!c || n_inst <= 0 || n_steps < 0 || !(h > 0) || !d_x_out || !d_inst_status)
    return fail(KRETS_ERR_INVALID_ARGUMENT, "invalid arguments to krets_batch_tran_noalloc");
  if ((d_values && !is_device_ptr(d_values)) || !is_device_ptr(d_x_out) || !is_device_ptr(d_inst_status))
    return fail(KRETS_ERR_INVALID_ARGUMENT, "krets_batch_tran_noalloc needs device pointers for values, "
                                            "x_out and inst_status");
  DevProgram *Ddc = find_program(c, MODE_DC, 0, 0, 0);
  DevProgram *Dtr = find_program(c, MODE_TRAN, method, h, 0);
  if (!Ddc || !Dtr)
    return fail(KRETS_ERR_INVALID_ARGUMENT, "krets_batch_tran_noalloc: the circuit has no compiled program for this "
                                            "time step and method; run krets_batch_tran once with them first");
  const DevProg &P = Dtr->view;
  const bool mixed = precision == KRETS_PREC_MIXED;
  // operating point: its per-CTA workspace must fit in shared memory (no global workspace)
  Lay Lop = layout_op(Ddc->view);
  if (Lop.bytes > max_smem_optin())
    return fail(KRETS_ERR_INVALID_ARGUMENT, "krets_batch_tran_noalloc: circuit too large for the shared-memory "
                                            "operating-point kernel");
  // warp engine layout (identical to krets_batch_tran's)
  WarpLay WL{};
  size_t cur = 0;
  auto put = [&](int &off, size_t bytes) { off = (int)cur; cur = align16(cur + bytes); };
  put(WL.lu, (mixed ? 4 : 8) * (size_t)P.nnz_lu);
  put(WL.coef, 8 * (size_t)P.ne);
  put(WL.x, 8 * (size_t)P.n);
  put(WL.b, 8 * (size_t)P.n);
  put(WL.w, mixed ? 4 * (size_t)P.n : 0);
  put(WL.cb, 8 * (size_t)P.ndyn);
  put(WL.icap, 8 * (size_t)P.ncap);
  put(WL.prev, P.nonlinear ? 8 * (size_t)P.n : 0);
  put(WL.guess, P.nonlinear ? 8 * (size_t)P.n : 0);
  WL.bytes = (int)align16(cur);
  WL.sprog_bytes = (int)align16((size_t)P.sp_off[11] * sizeof(int));
  const size_t per_warp = WL.bytes;
  if (!P.sprog_ok || per_warp + WL.sprog_bytes > max_smem_optin())
    return fail(KRETS_ERR_INVALID_ARGUMENT, "krets_batch_tran_noalloc: circuit too large for the warp engine");
  int W = (int)std::max<size_t>(1, std::min<size_t>(8, (max_smem_optin() - WL.sprog_bytes) / per_warp));
  const size_t smem = WL.sprog_bytes + (size_t)W * per_warp;
  auto kern = mixed ? k_tran_warp<1> : k_tran_warp<0>;
  CU(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32 * W, smem));
  if (per_sm < 1) return fail(KRETS_ERR_CUDA, "warp engine does not fit on an SM");
  int grid = std::max(1, std::min((n_inst + W - 1) / W, per_sm * device_sm_count()));
  // scratch layout: [0,64) counters, [64,128) histogram, [256, 256+4n) OP status, then the
  // FP64 fallback factors of every warp slot (mixed precision)
  const size_t op_off = 256;
  const size_t lu_off = align16(op_off + sizeof(int) * (size_t)n_inst);
  const size_t lu_slot = sizeof(double) * (size_t)P.nnz_lu;
  if (lu_off > KRETS_NOALLOC_SCRATCH_BYTES)
    return fail(KRETS_ERR_INVALID_ARGUMENT, "krets_batch_tran_noalloc: too many instances for the 16 MiB scratch");
  if (mixed) {
    const size_t slots = (KRETS_NOALLOC_SCRATCH_BYTES - lu_off) / lu_slot;
    if (slots < (size_t)W)
      return fail(KRETS_ERR_INVALID_ARGUMENT, "krets_batch_tran_noalloc: instance size exceeds the 16 MiB scratch");
    grid = std::min(grid, (int)(slots / W));
  }
  void *scr = nullptr;
  krets_status s = noalloc_scratch_address(&scr);
  if (s) return s;
  char *base = (char *)scr;
  int *queue = (int *)(base + 0);
  int *fallbacks = (int *)(base + 4);
  int *any = (int *)(base + 8);
  unsigned long long *hist = (unsigned long long *)(base + 64);
  int *op_status = (int *)(base + op_off);
  double *fb = mixed ? (double *)(base + lu_off) : nullptr;
  CU(cudaEventRecord(c->ev[0], c->stream));
  // everything that must start at zero: counters, histogram, statuses
  CU(cudaMemsetAsync(base, 0, 256, c->stream));
  CU(cudaMemsetAsync(op_status, 0, sizeof(int) * (size_t)n_inst, c->stream));
  CU(cudaMemsetAsync(d_inst_status, 0, sizeof(int) * (size_t)n_inst, c->stream));
  const size_t stride = (size_t)c->n * ((size_t)n_steps + 1);
  int op_grid;
  size_t op_smem;
  char *op_gws;
  s = plan_launch(c, k_op, Lop, 128, n_inst, op_grid, op_smem, op_gws);
  if (s) return s;
  k_op<<<op_grid, 128, op_smem, c->stream>>>(Ddc->view, c->cfg, Lop, nullptr, d_values, d_x_out, stride, op_status,
                                             nullptr, n_inst);
  g_launches++;
  CU(cudaGetLastError());
  const char *tenv = getenv("KRETS_REFINE_TOL");
  const double tol = tenv ? atof(tenv) : 1e-10;
  CU(cudaEventRecord(c->ev[2], c->stream));
  kern<<<grid, 32 * W, smem, c->stream>>>(P, c->cfg, WL, d_values, n_inst, h, n_steps, method, source_lag, d_x_out,
                                         d_inst_status, queue, hist, fallbacks, fb, tol);
  g_launches++;
  CU(cudaGetLastError());
  CU(cudaEventRecord(c->ev[3], c->stream));
  k_status_fold<<<std::max(1, std::min(1024, (n_inst + 255) / 256)), 256, 0, c->stream>>>(op_status, d_inst_status,
                                                                                         n_inst, any);
  g_launches++;
  CU(cudaGetLastError());
  int any_h = 0;
  CU(cudaMemcpyAsync(&any_h, any, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  CU(cudaEventRecord(c->ev[1], c->stream));
  CU(cudaStreamSynchronize(c->stream));
  cudaEventElapsedTime(&c->kernel_ms, c->ev[2], c->ev[3]);
  cudaEventElapsedTime(&c->call_ms, c->ev[0], c->ev[1]);
  return map_status(any_h, 1);
}

}  // extern "C"
