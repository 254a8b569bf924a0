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
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "kernels.cuh"
#include "warp_kernels.cuh"
#include "adjoint.cuh"
#include "multi.cuh"
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

size_t max_smem_per_sm() {
  static int v = -1;
  if (v < 0) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) != cudaSuccess)
      v = 64 * 1024;
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

// Host memory that is page-locked (cudaHostAlloc or cudaHostRegister) over [p, p + bytes).
bool is_pinned_host(const void *p, size_t bytes) {
  if (!p || !bytes) return false;
  for (const char *q : {(const char *)p, (const char *)p + bytes - 1}) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, q) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    if (a.type != cudaMemoryTypeHost) return false;
  }
  return true;
}

// Kernels may read and write pageable host memory directly on systems whose GPU shares the
// host's page tables (Grace: NVLink-C2C with address translation); then host buffers are
// used in place instead of through a device copy.  KRETS_NO_DIRECT_HOST=1 turns it off.
bool direct_host_access() {
  static int cached = -1;
  if (cached < 0) {
    int dev = 0, v = 0;
    cached = 0;
    const char *off = getenv("KRETS_NO_DIRECT_HOST");
    if (!(off && off[0] == '1') && cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) == cudaSuccess)
      cached = v ? 1 : 0;
    cudaGetLastError();
  }
  return cached == 1;
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
  // status words of single solves in mapped pinned host memory (host and device address):
  // the kernel writes them where the host reads them, so a call needs no copy for them
  int *h_small = nullptr, *h_small_dev = nullptr;
  unsigned long long *d_hist = nullptr;
  long long hist[8] = {};
  int fallbacks = 0;
  int warps_per_cta = 0, grid = 0;
  int launch_info[5] = {0, 0, 0, 0, 0};  // last batched launch: threads per instance, per CTA, grid, tuned, lug
  void *l2buf = nullptr;
  // global-memory factors of the double-float engine's groups (k_tran_dfd<G, true>)
  void *lug = nullptr;
  size_t lug_bytes = 0;
  // per-CTA coefficient cache of the batched AC sweep (k_ac_batch<1>)
  void *accache = nullptr;
  size_t accache_bytes = 0;
  // staged host output of the double-float engine: two staging buffers, a copy stream
  void *stage = nullptr;
  size_t stage_bytes = 0;
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t sev[5] = {};  // kernel done x2, copy done x2, operating point done

  ~krets_circuit() {
    if (lug) cudaFree(lug);
    if (accache) cudaFree(accache);
    if (stage) cudaFree(stage);
    for (auto &e : sev)
      if (e) cudaEventDestroy(e);
    if (copy_stream) cudaStreamDestroy(copy_stream);
    if (d_el) cudaFree(d_el);
    if (scratch) cudaFree(scratch);
    if (d_small) cudaFree(d_small);
    if (h_small) cudaFreeHost(h_small);
    if (d_hist) cudaFree(d_hist);
    if (l2buf) cudaFree(l2buf);
    for (auto &e : ev)
      if (e) cudaEventDestroy(e);
    if (stream) cudaStreamDestroy(stream);
  }

  krets_status ensure_lug(size_t bytes) {
    if (bytes <= lug_bytes) return KRETS_OK;
    if (lug) cudaFree(lug);
    lug = nullptr;
    lug_bytes = 0;
    CU(cudaMalloc(&lug, bytes));
    lug_bytes = bytes;
    return KRETS_OK;
  }

  krets_status ensure_stage(size_t bytes) {
    if (!copy_stream) {
      CU(cudaStreamCreateWithFlags(&copy_stream, cudaStreamNonBlocking));
      for (auto &e : sev) CU(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    if (bytes <= stage_bytes) return KRETS_OK;
    if (stage) cudaFree(stage);
    stage = nullptr;
    stage_bytes = 0;
    CU(cudaMalloc(&stage, bytes));
    stage_bytes = bytes;
    return KRETS_OK;
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

// Device image of a program: every array at a 16-byte aligned offset of one buffer.
// program_bytes() sizes it; place_program() writes the arrays into a host staging copy of
// that buffer (host_base) and sets the view's pointers into its device copy (dev_base).
struct ProgramImage {
  std::vector<int> lu_src, is_cur;
};

static void image_extras(const Program &H, ProgramImage &X) {
  X.lu_src.assign(H.lu_col.size(), -1);
  for (size_t t = 0; t < H.a_slot.size(); ++t) X.lu_src[H.a_slot[t]] = (int)t;
  X.is_cur.assign(H.n, 0);
  for (int e = 0; e < H.ne; ++e)
    if (H.el_pos[4 * e + 2] >= 0) X.is_cur[H.el_pos[4 * e + 2]] = 1;
}

template <typename F>
static void for_each_array(const Program &H, const ProgramImage &X, F &&f) {
  f(H.q); f(H.lu_rowptr); f(H.lu_col); f(H.lu_diag); f(X.lu_src);
  f(H.a_rowptr); f(H.a_col); f(H.a_cptr); f(H.a_contrib);
  f(H.b_cptr); f(H.b_contrib); f(H.piv_ptr); f(H.piv); f(H.upd);
  f(H.lev_ptr); f(H.lev_rows); f(H.ulev_ptr); f(H.ulev_rows);
  f(H.el_pos); f(X.is_cur);
  f(H.qinv); f(H.ldesc); f(H.udesc); f(H.res_ptr); f(H.res_op);
  f(H.dyn_e); f(H.bd_ptr); f(H.bd_op); f(H.sprog);
  f(H.tprog); f(H.prow); f(H.xslot); f(H.iprog); f(H.imap);
}

static size_t program_bytes(const Program &H, const ProgramImage &X) {
  size_t total = 0;
  for_each_array(H, X, [&](const std::vector<int> &v) { total = align16(total + (v.empty() ? 4 : v.size() * 4)); });
  return total;
}

static void place_program(const Program &H, const ProgramImage &X, const krets_element *el_host,
                          const krets_element *d_el, char *dev_base, char *host_base, DevProg &V) {
  std::vector<const void *> p;
  size_t off = 0;
  for_each_array(H, X, [&](const std::vector<int> &v) {
    if (!v.empty()) memcpy(host_base + off, v.data(), v.size() * 4);
    p.push_back(dev_base + off);
    off = align16(off + (v.empty() ? 4 : v.size() * 4));
  });
  size_t i = 0;
  auto nx = [&]() { return p[i++]; };
  V.n = H.n;
  V.ne = H.ne;
  V.nnz_a = (int)H.a_col.size();
  V.nnz_lu = (int)H.lu_col.size();
  V.nlev = (int)H.lev_ptr.size() - 1;
  V.nulev = (int)H.ulev_ptr.size() - 1;
  V.mode = H.mode;
  V.method = H.method;
  V.q = (const int *)nx();
  V.lu_rowptr = (const int *)nx();
  V.lu_col = (const int *)nx();
  V.lu_diag = (const int *)nx();
  V.lu_src = (const int *)nx();
  V.a_rowptr = (const int *)nx();
  V.a_col = (const int *)nx();
  V.a_cptr = (const int *)nx();
  V.a_contrib = (const int *)nx();
  V.b_cptr = (const int *)nx();
  V.b_contrib = (const int *)nx();
  V.piv_ptr = (const int *)nx();
  V.piv = (const int4 *)nx();
  V.upd = (const int2 *)nx();
  V.lev_ptr = (const int *)nx();
  V.lev_rows = (const int *)nx();
  V.ulev_ptr = (const int *)nx();
  V.ulev_rows = (const int *)nx();
  V.el_pos = (const int4 *)nx();
  V.is_cur = (const int *)nx();
  V.qinv = (const int *)nx();
  V.ldesc = (const int4 *)nx();
  V.udesc = (const int4 *)nx();
  V.res_ptr = (const int *)nx();
  V.res_op = (const int2 *)nx();
  V.dyn_e = (const int *)nx();
  V.bd_ptr = (const int *)nx();
  V.bd_op = (const int *)nx();
  V.sprog = (const int *)nx();
  V.tprog = (const int *)nx();
  V.prow = (const int *)nx();
  V.xslot = (const int *)nx();
  V.iprog = (const int *)nx();
  V.imap = (const int *)nx();
  for (int gi = 0; gi < 3; ++gi) {
    for (int k = 0; k < 4; ++k) V.ip_off[gi][k] = H.ip_off[gi][k];
    V.il_slots[gi] = H.il_slots[gi];
    V.imap_off[gi] = H.imap_off[gi];
  }
  V.n_il_lrec = H.n_il_lrec;
  V.n_il_urec = H.n_il_urec;
  V.il_ok = H.il_ok ? 1 : 0;
  V.lean_off = H.lean_off;
  V.n_zrow = H.n_zrow;
  V.n_ind = H.n_ind;
  V.lean_ok = H.lean_ok ? 1 : 0;
  V.n_coef = H.n_coef;
  V.el = d_el;
  V.ndyn = (int)H.dyn_e.size();
  V.ncap = H.ncap;
  V.n_resop = (int)H.res_op.size() / 2;
  for (int k = 0; k < 16; ++k) V.sp_off[k] = H.sp_off[k];
  V.n_bchunk = H.n_bchunk;
  V.n_brow = H.n_brow;
  V.sprog_ok = H.sprog_ok;
  for (int k = 0; k < 8; ++k) V.tp_off[k] = H.tp_off[k];
  V.n_utlev = H.n_utlev;
  V.n_ltlev = H.n_ltlev;
  V.tail0 = H.tail0;
  V.tail_m = H.tail_m;
  bool nl = false;
  for (int e = 0; e < H.ne; ++e) {
    int k = el_host[e].kind;
    if (H.mode == MODE_DC && k == KRETS_ELEM_C) continue;
    if (k == KRETS_ELEM_D || k == KRETS_ELEM_M || k == KRETS_ELEM_Q) nl = true;
  }
  V.nonlinear = nl;
}

krets_status upload_program(krets_circuit *c, Program &&P, DevProgram &D) {
  D.host = std::move(P);
  ProgramImage X;
  image_extras(D.host, X);
  const size_t total = program_bytes(D.host, X);
  CU(cudaMalloc(&D.buf, total));
  std::vector<char> staging(total, 0);
  place_program(D.host, X, c->el.data(), c->d_el, (char *)D.buf, staging.data(), D.view);
  CU(cudaMemcpy(D.buf, staging.data(), total, cudaMemcpyHostToDevice));
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
  B.add(4, sizeof(double) * P.n_coef);
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
  B.add(8, sizeof(double) * P.n_coef);
  B.add(9, sizeof(double) * P.ne);
  B.add(10, sizeof(double) * P.ne);
  B.add(11, sizeof(double) * 32);
  B.add(12, sizeof(int) * 4);
  B.add(13, sizeof(int) * 4);
  return B.done();
}

Lay layout_adaptive(const DevProg &P) {
  LayBuilder B;
  B.add(0, sizeof(double) * P.ne);
  B.add(1, sizeof(double) * P.nnz_lu);
  B.add(2, sizeof(double) * P.n);
  B.add(3, sizeof(double) * P.n);
  B.add(4, sizeof(double) * P.n);
  B.add(5, sizeof(double) * P.n_coef);
  B.add(6, sizeof(double) * P.ne);
  B.add(7, sizeof(double) * P.ne);
  B.add(8, sizeof(double) * 32);
  B.add(9, sizeof(int) * 4);
  B.add(10, sizeof(double) * P.n);
  return B.done();
}

// MIXED: the stamping pass's coefficient arrays (slots 6, 7, 8) are dead once the
// complex128 matrix and the rhs are summed, so the complex64 LU, the correction and the
// solution (slots 2, 5, 3) reuse their bytes; the element values (slot 0) are read from
// the caller's array.  That keeps a CTA of the 500-section ladder near 68 KB, three per SM.
Lay layout_ac(const DevProg &P, bool mixed) {
  if (mixed) {
    LayBuilder B;
    B.add(1, 16 * (size_t)P.nnz_a);
    B.add(4, 16 * (size_t)P.n);
    B.add(9, sizeof(double) * P.n);
    B.add(10, sizeof(double) * 32);
    B.add(11, sizeof(int) * 4);
    B.add(12, sizeof(int) * 4);
    const size_t r0 = B.cur;
    B.add(6, sizeof(double) * P.n_coef);
    B.add(7, sizeof(double) * P.n_coef);
    B.add(8, sizeof(double) * P.ne);
    const size_t r1 = B.cur;
    B.cur = r0;
    B.add(2, 8 * (size_t)P.nnz_lu);
    B.add(5, 8 * (size_t)P.n);
    B.add(3, 16 * (size_t)P.n);
    B.cur = std::max(B.cur, r1);
    B.L.off[0] = -1;
    return B.done();
  }
  LayBuilder B;
  B.add(0, sizeof(double) * P.ne);
  B.add(1, mixed ? 16 * (size_t)P.nnz_a : 0);
  B.add(2, (mixed ? 8 : 16) * (size_t)P.nnz_lu);
  B.add(3, 16 * (size_t)P.n);
  B.add(4, 16 * (size_t)P.n);
  B.add(5, mixed ? 8 * (size_t)P.n : 0);
  B.add(6, sizeof(double) * P.n_coef);
  B.add(7, sizeof(double) * P.n_coef);
  B.add(8, sizeof(double) * P.ne);
  B.add(9, sizeof(double) * P.n);
  B.add(10, sizeof(double) * 32);
  B.add(11, sizeof(int) * 4);
  B.add(12, sizeof(int) * 4);
  return B.done();
}

// Resident CTAs per SM of a kernel at a block size and dynamic shared memory, with the
// kernel's shared-memory limit raised to that size.  Both runtime queries cost
// microseconds, which a single-solve call would pay every time, so the answers are kept
// per (device, kernel, block size, shared memory); the limit is only ever raised.
template <typename K>
krets_status kernel_fit(K kernel, int threads, size_t smem, int &per_sm) {
  struct Fit { int dev; const void *k; int threads; size_t smem; int per_sm; };
  struct Limit { int dev; const void *k; size_t smem; };
  static std::mutex mu;
  static std::vector<Fit> fits;
  static std::vector<Limit> limits;
  int dev = 0;
  CU(cudaGetDevice(&dev));
  const void *k = reinterpret_cast<const void *>(kernel);
  std::lock_guard<std::mutex> lock(mu);
  for (const Fit &f : fits)
    if (f.dev == dev && f.k == k && f.threads == threads && f.smem == smem) {
      per_sm = f.per_sm;
      return KRETS_OK;
    }
  Limit *lim = nullptr;
  for (Limit &l : limits)
    if (l.dev == dev && l.k == k) lim = &l;
  if (!lim || lim->smem < smem) {
    CU(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    if (lim) lim->smem = smem;
    else limits.push_back(Limit{dev, k, smem});
  }
  CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem));
  fits.push_back(Fit{dev, k, threads, smem, per_sm});
  return KRETS_OK;
}

// Decide shared vs global placement and the grid for a per-CTA workspace.
template <typename K>
krets_status plan_launch(krets_circuit *c, K kernel, const Lay &L, int threads, int items, int &grid,
                         size_t &smem, char *&gws) {
  if (L.bytes <= max_smem_optin()) {
    smem = L.bytes;
    gws = nullptr;
    int per_sm = 0;
    krets_status s = kernel_fit(kernel, threads, smem, per_sm);
    if (s != KRETS_OK) return s;
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
  if (bits & KS_TSTEP) return fail(KRETS_ERR_UNEXPECTED, "time step fell below h_min");
  if (bits & KS_FULL) return fail(KRETS_ERR_INVALID_ARGUMENT, "more accepted time points than max_points");
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
  if (is_device_ptr(user) || direct_host_access()) {
    *dptr = const_cast<void *>(user);
    return KRETS_OK;
  }
  CU(cudaMalloc(&tmp.p, bytes));
  if (in) CU(cudaMemcpyAsync(tmp.p, user, bytes, cudaMemcpyHostToDevice, s));
  *dptr = tmp.p;
  return KRETS_OK;
}

// Program arrays a launch of at most one CTA per SM warms into L1 (see warm_l1):
// factorisation, solves, then stamps; only the stamps when the first group is staged in
// shared memory (plan_stage).  Empty when CTAs share SMs.
OpWarm plan_warm(const DevProgram *D, int n_inst, bool staged = false) {
  OpWarm w{};
  if (n_inst > device_sm_count()) return w;
  const DevProg &V = D->view;
  const Program &H = D->host;
  const struct { const void *p; size_t words; bool fac; } fs[] = {
      {V.piv_ptr, H.piv_ptr.size(), true},    {V.piv, H.piv.size(), true},
      {V.upd, H.upd.size(), true},            {V.lu_diag, H.lu_diag.size(), true},
      {V.lev_rows, H.lev_rows.size(), true},  {V.lu_rowptr, H.lu_rowptr.size(), true},
      {V.lu_col, H.lu_col.size(), true},      {V.ulev_rows, H.ulev_rows.size(), true},
      {V.lu_src, H.lu_col.size(), false},     {V.a_cptr, H.a_cptr.size(), false},
      {V.a_contrib, H.a_contrib.size(), false}, {V.b_cptr, H.b_cptr.size(), false},
      {V.b_contrib, H.b_contrib.size(), false}};
  for (const auto &f : fs) {
    if (f.words == 0 || w.count == 16 || (staged && f.fac)) continue;
    w.ptr[w.count] = static_cast<const char *>(f.p);
    w.bytes[w.count] = (int)(4 * f.words);
    ++w.count;
  }
  return w;
}

// Shared-memory copies of the factorisation and solve arrays (see stage_fac) for launches
// of at most one CTA per SM whose workspace leaves room for them; L.bytes grows by the
// staged region, so the launch sizes its dynamic shared memory for both.
OpStage plan_stage(const DevProgram *D, int n_inst, Lay &L) {
  OpStage S{};
  if (n_inst > device_sm_count()) return S;
  const Program &H = D->host;
  const size_t words[10] = {H.lev_ptr.size(),   H.lev_rows.size(), H.piv_ptr.size(),   H.lu_diag.size(),
                            H.lu_rowptr.size(), H.lu_col.size(),   H.ulev_ptr.size(),  H.ulev_rows.size(),
                            H.piv.size(),       H.upd.size()};
  const size_t off = align16(L.bytes);
  size_t at = 0;
  for (int a = 0; a < 10; ++a) {
    const size_t n16 = (words[a] * 4 + 15) / 16;
    S.at[a] = (int)at;
    S.n16[a] = (int)n16;
    at += 16 * n16;
  }
  if (off + at > (size_t)max_smem_optin()) return OpStage{};
  S.on = 1;
  S.off = (int)off;
  L.bytes = off + at;
  return S;
}

krets_status run_op(krets_circuit *c, DevProgram *D, int n_inst, const double *d_values, double *d_x,
                    size_t out_stride, int *d_status, int *d_iters, int threads) {
  Lay L = layout_op(D->view);
  int grid;
  size_t smem;
  char *gws;
  const OpStage stage = plan_stage(D, n_inst, L);
  krets_status s = plan_launch(c, k_op, L, threads, n_inst, grid, smem, gws);
  if (s != KRETS_OK) return s;
  k_op<<<grid, threads, smem, c->stream>>>(D->view, c->cfg, L, gws, d_values, d_x, out_stride, d_status, d_iters,
                                          n_inst, plan_warm(D, n_inst, stage.on), stage);
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

// Device address of g_noalloc_scratch per device, looked up once per device with that
// device current (the host-side name of the array is only a stand-in, never a device
// address).  Atomic slots: two host threads making their first call on one device at the
// same time may both look it up, and both store the same address.
constexpr int kMaxDevices = 64;
std::atomic<void *> g_noalloc_addr[kMaxDevices];

krets_status noalloc_scratch_address(void **out) {
  int dev = 0;
  CU(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return fail(KRETS_ERR_CUDA, "device index out of range");
  void *p = g_noalloc_addr[dev].load(std::memory_order_acquire);
  if (!p) {
    CU(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    g_noalloc_addr[dev].store(p, std::memory_order_release);
  }
  *out = p;
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
// status array, plus one summary word for each (the operating point's failures map to
// the operating-point error codes, as in krets_batch_tran).
__global__ void k_status_fold(const int *op_status, int *inst_status, int n, int *any_op, int *any_tran) {
  int acc_op = 0, acc_tr = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int o = op_status[i], t = inst_status[i];
    inst_status[i] = o | t;
    acc_op |= o;
    acc_tr |= t;
  }
  if (acc_op) atomicOr(any_op, acc_op);
  if (acc_tr) atomicOr(any_tran, acc_tr);
}

}  // namespace

// ====================================================================== C ABI
// Many distinct circuits run by one multi-circuit launch set (krets_multi_*).
struct MultiClass {
  int G = 0, W = 0;          // group size, groups per CTA
  bool global = false;       // working arrays in global memory
  long long region = 0;      // bytes per group
  std::vector<int> items;    // circuits, largest first
  int grid = 0;
  long long gsm = 0;         // global class: shared memory per group
  bool x_smem = false;       // global class: solution and rhs coefficients in shared memory
  float ms = 0.f;            // last run: launch set start to this class's end
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
};

struct krets_multi {
  int n_circ = 0, method = 0;
  double h = 0;
  std::vector<int> n, ne;
  std::vector<long long> el_off;
  krets_element *d_el = nullptr;
  void *d_image = nullptr;  // every program's arrays
  DevProg *d_views = nullptr;  // [2 * n_circ]: DC, TRAN
  std::vector<long long> nnz_lu_tr, levels_tr;
  std::vector<MultiClass> classes;
  int *d_queue = nullptr, *d_status = nullptr;
  long long *d_xoff = nullptr;
  int *d_items = nullptr;
  char *gscratch = nullptr;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[4] = {};
  float kernel_ms = 0.f, call_ms = 0.f;
  ~krets_multi() {
    for (auto &k : classes) {
      if (k.stream) cudaStreamDestroy(k.stream);
      if (k.done) cudaEventDestroy(k.done);
    }
    for (auto p : {(void *)d_el, d_image, (void *)d_views, (void *)d_queue, (void *)d_status, (void *)d_xoff,
                   (void *)d_items, (void *)gscratch})
      if (p) cudaFree(p);
    for (auto &e : ev)
      if (e) cudaEventDestroy(e);
    if (stream) cudaStreamDestroy(stream);
  }
};

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
  if (!c->h_small) {
    void *hp = nullptr, *dp = nullptr;
    CU(cudaHostAlloc(&hp, 64, cudaHostAllocMapped));
    c->h_small = static_cast<int *>(hp);
    CU(cudaHostGetDevicePointer(&dp, hp, 0));
    c->h_small_dev = static_cast<int *>(dp);
  }
  // the previous call on this stream has finished (it synchronised), so nothing writes these
  volatile int *h = c->h_small;
  h[0] = 0;
  h[1] = 0;
  CU(cudaEventRecord(c->ev[0], c->stream));
  s = dev_view(x_out, sizeof(double) * c->n, false, c->stream, tx, &dx);
  if (s) return s;
  CU(cudaEventRecord(c->ev[2], c->stream));
  s = run_op(c, D, 1, nullptr, (double *)dx, c->n, c->h_small_dev, c->h_small_dev + 1, plain_threads(D->view));
  if (s) return s;
  CU(cudaEventRecord(c->ev[3], c->stream));
  if (tx.p) CU(cudaMemcpyAsync(x_out, dx, sizeof(double) * c->n, cudaMemcpyDeviceToHost, c->stream));
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

namespace {

// Shared by krets_dc and krets_batch_dc: checks the sweep and returns its point count
// (|(stop-start)/step| + 1, truncated: dc.rs:153-154).
krets_status dc_points(krets_circuit *c, int32_t sweep_elem, double start, double stop, double step, int &np) {
  if (sweep_elem < 0 || sweep_elem >= c->ne) return fail(KRETS_ERR_ELEMENT_NOT_FOUND, "sweep element not found");
  int kind = c->el[sweep_elem].kind;
  if (kind != KRETS_ELEM_V && kind != KRETS_ELEM_I)
    return fail(KRETS_ERR_INVALID_ELEMENT, "DC sweep element must be a voltage or current source");
  double np_d = std::fabs((stop - start) / step);
  if (!(np_d < 1e9)) return fail(KRETS_ERR_INVALID_ARGUMENT, "invalid sweep range");
  np = (int)np_d + 1;
  return KRETS_OK;
}

krets_status run_dc(krets_circuit *c, int32_t sweep_elem, double start, double step, int np, int n_inst,
                    const double *values, double *x_out, int *d_status) {
  DevProgram *D;
  krets_status s = get_program(c, MODE_DC, 0, 0, 0, &D);
  if (s != KRETS_OK) return s;
  const size_t out_bytes = sizeof(double) * c->n * (size_t)np * n_inst;
  DevBuf tv, tx;
  void *dv, *dx;
  s = dev_view(values, sizeof(double) * c->ne * (size_t)n_inst, true, c->stream, tv, &dv);
  if (s) return s;
  s = dev_view(x_out, out_bytes, false, c->stream, tx, &dx);
  if (s) return s;
  Lay L = layout_op(D->view);
  int threads = plain_threads(D->view), grid;
  size_t smem;
  char *gws;
  const OpStage stage = plan_stage(D, n_inst, L);
  s = plan_launch(c, k_dc_sweep, L, threads, n_inst, grid, smem, gws);
  if (s) return s;
  CU(cudaEventRecord(c->ev[2], c->stream));
  k_dc_sweep<<<grid, threads, smem, c->stream>>>(D->view, c->cfg, L, gws, sweep_elem, start, step, np,
                                                 (const double *)dv, n_inst, (size_t)c->n * np, (double *)dx,
                                                 d_status, plan_warm(D, n_inst, stage.on), stage);
  g_launches++;
  CU(cudaGetLastError());
  CU(cudaEventRecord(c->ev[3], c->stream));
  if (tx.p) CU(cudaMemcpyAsync(x_out, dx, out_bytes, cudaMemcpyDeviceToHost, c->stream));
  return KRETS_OK;
}

}  // namespace

krets_status krets_dc(krets_circuit *c, int32_t sweep_elem, double start, double stop, double step, double *x_out,
                      int32_t max_points, int32_t *n_points) {
  if (!c || !x_out) return fail(KRETS_ERR_INVALID_ARGUMENT, "null argument");
  int np;
  krets_status s = dc_points(c, sweep_elem, start, stop, step, np);
  if (s != KRETS_OK) return s;
  if (n_points) *n_points = np;
  if (np > max_points) return fail(KRETS_ERR_INVALID_ARGUMENT, "x_out too small for the sweep");
  CU(cudaEventRecord(c->ev[0], c->stream));
  s = run_dc(c, sweep_elem, start, step, np, 1, nullptr, x_out, c->d_small);
  if (s != KRETS_OK) return s;
  int h = 0;
  CU(cudaMemcpyAsync(&h, c->d_small, sizeof h, cudaMemcpyDeviceToHost, c->stream));
  CU(cudaEventRecord(c->ev[1], c->stream));
  CU(cudaStreamSynchronize(c->stream));
  cudaEventElapsedTime(&c->kernel_ms, c->ev[2], c->ev[3]);
  cudaEventElapsedTime(&c->call_ms, c->ev[0], c->ev[1]);
  return map_status(h, 1);
}

krets_status krets_batch_dc(krets_circuit *c, int32_t n_inst, const double *values, int32_t sweep_elem,
                            double start, double stop, double step, double *x_out, int32_t max_points,
                            int32_t *n_points, int32_t *inst_status) {
  if (!c || !x_out || n_inst <= 0) return fail(KRETS_ERR_INVALID_ARGUMENT, "invalid arguments");
  int np;
  krets_status s = dc_points(c, sweep_elem, start, stop, step, np);
  if (s != KRETS_OK) return s;
  if (n_points) *n_points = np;
  if (np > max_points) return fail(KRETS_ERR_INVALID_ARGUMENT, "x_out too small for the sweep");
  CU(cudaEventRecord(c->ev[0], c->stream));
  DevBuf ts;
  CU(cudaMalloc(&ts.p, sizeof(int) * n_inst));
  CU(cudaMemsetAsync(ts.p, 0, sizeof(int) * n_inst, c->stream));
  s = run_dc(c, sweep_elem, start, step, np, n_inst, values, x_out, (int *)ts.p);
  if (s != KRETS_OK) return s;
  std::vector<int> st(n_inst);
  CU(cudaMemcpyAsync(st.data(), ts.p, sizeof(int) * n_inst, cudaMemcpyDeviceToHost, c->stream));
  CU(cudaEventRecord(c->ev[1], c->stream));
  CU(cudaStreamSynchronize(c->stream));
  cudaEventElapsedTime(&c->kernel_ms, c->ev[2], c->ev[3]);
  cudaEventElapsedTime(&c->call_ms, c->ev[0], c->ev[1]);
  int any = 0;
  for (int i = 0; i < n_inst; ++i) {
    if (inst_status) inst_status[i] = st[i];
    any |= st[i];
  }
  return map_status(any, 1);
}

krets_status krets_batch_tran_adaptive(krets_circuit *c, int32_t n_inst, const double *values, double h0,
                                       double t_stop, int32_t method, double lte_tol, double h_min, double h_max,
                                       int32_t max_points, double *t_out, double *x_out, int32_t *n_points,
                                       int32_t *inst_status) {
  if (!c || !t_out || !x_out || !n_points || n_inst <= 0 || max_points < 2 || !(h0 > 0) || !(t_stop > 0) ||
      !(lte_tol > 0) || !(h_min > 0) || !(h_min <= h0) || !(h_max >= h0) ||
      (method != KRETS_METHOD_BE && method != KRETS_METHOD_TR))
    return fail(KRETS_ERR_INVALID_ARGUMENT, "invalid arguments to krets_batch_tran_adaptive");
  DevProgram *Ddc, *Dtr;
  krets_status s = get_program(c, MODE_DC, 0, 0, 0, &Ddc);
  if (s != KRETS_OK) return s;
  s = get_program(c, MODE_TRAN, method, h0, 0, &Dtr);  // pivots chosen at h0
  if (s != KRETS_OK) return s;
  CU(cudaEventRecord(c->ev[0], c->stream));
  const size_t stride = (size_t)c->n * max_points;
  DevBuf tv, tx, tt, tn, ts;
  void *dv, *dx, *dt, *dn;
  s = dev_view(values, sizeof(double) * c->ne * (size_t)n_inst, true, c->stream, tv, &dv);
  if (s) return s;
  s = dev_view(x_out, sizeof(double) * stride * n_inst, false, c->stream, tx, &dx);
  if (s) return s;
  s = dev_view(t_out, sizeof(double) * (size_t)max_points * n_inst, false, c->stream, tt, &dt);
  if (s) return s;
  s = dev_view(n_points, sizeof(int) * (size_t)n_inst, false, c->stream, tn, &dn);
  if (s) return s;
  CU(cudaMalloc(&ts.p, sizeof(int) * 2 * (size_t)n_inst));
  int *d_st = (int *)ts.p, *d_opst = d_st + n_inst;
  CU(cudaMemsetAsync(ts.p, 0, sizeof(int) * 2 * (size_t)n_inst, c->stream));
  CU(cudaEventRecord(c->ev[2], c->stream));
  s = run_op(c, Ddc, n_inst, (const double *)dv, (double *)dx, stride, d_opst, nullptr, 128);
  if (s) return s;
  const DevProg &P = Dtr->view;
  Lay L = layout_adaptive(P);
  int threads = plain_threads(P), grid;
  size_t smem;
  char *gws;
  s = plan_launch(c, k_tran_adaptive, L, threads, n_inst, grid, smem, gws);
  if (s) return s;
  k_tran_adaptive<<<grid, threads, smem, c->stream>>>(P, c->cfg, L, gws, (const double *)dv, n_inst, h0, t_stop,
                                                      method, lte_tol, h_min, h_max, max_points, (double *)dt,
                                                      (double *)dx, (int *)dn, d_st);
  g_launches++;
  CU(cudaGetLastError());
  CU(cudaEventRecord(c->ev[3], c->stream));
  if (tx.p) CU(cudaMemcpyAsync(x_out, dx, sizeof(double) * stride * n_inst, cudaMemcpyDeviceToHost, c->stream));
  if (tt.p) CU(cudaMemcpyAsync(t_out, dt, sizeof(double) * max_points * (size_t)n_inst, cudaMemcpyDeviceToHost, c->stream));
  if (tn.p) CU(cudaMemcpyAsync(n_points, dn, sizeof(int) * (size_t)n_inst, cudaMemcpyDeviceToHost, c->stream));
  std::vector<int> st(2 * (size_t)n_inst);
  CU(cudaMemcpyAsync(st.data(), d_st, sizeof(int) * 2 * (size_t)n_inst, cudaMemcpyDeviceToHost, c->stream));
  CU(cudaEventRecord(c->ev[1], c->stream));
  CU(cudaStreamSynchronize(c->stream));
  cudaEventElapsedTime(&c->kernel_ms, c->ev[2], c->ev[3]);
  cudaEventElapsedTime(&c->call_ms, c->ev[0], c->ev[1]);
  int any = 0;
  for (int i = 0; i < n_inst; ++i) {
    const int v = st[i] | st[n_inst + i];
    if (inst_status) inst_status[i] = v;
    any |= v;
  }
  return map_status(any, 0);
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
  // one complex system per CTA, latency bound: 256 threads (for n >= 256; measured on the
  // 500-section ladder, three CTAs per SM: 128 threads 2.61e6, 256 2.87e6, 384 2.91e6, 512
  // 2.60e6 points/s)
  int threads = Dac->view.n >= 256 ? 256 : 128, grid;
  size_t smem;
  char *gws;
  auto kern = mixed ? k_ac_batch<1> : k_ac_batch<0>;
  s = plan_launch(c, kern, L, threads, (int)std::min<size_t>(items, 1 << 30), grid, smem, gws);
  if (s) return s;
  int *queue = c->d_small + 8;
  CU(cudaMemsetAsync(queue, 0, sizeof(int), c->stream));
  // per-CTA cache of the frequency-independent coefficients (complex64 path), kept in the
  // handle across calls
  if (mixed) {
    const size_t bytes = sizeof(double) * (size_t)grid * (2 * (size_t)Dac->view.n_coef + Dac->view.ne);
    if (bytes > c->accache_bytes) {
      if (c->accache) cudaFree(c->accache);
      c->accache = nullptr;
      c->accache_bytes = 0;
      CU(cudaMalloc(&c->accache, bytes));
      c->accache_bytes = bytes;
    }
  }
  CU(cudaEventRecord(c->ev[2], c->stream));
  kern<<<grid, threads, smem, c->stream>>>(Dac->view, L, gws, (const double *)dv, (const double *)top.p, n_inst,
                                           (const double *)df, n_freq, (double *)dx, d_item_st, queue,
                                           mixed ? (double *)c->accache : nullptr);
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
  size_t nd = 8 * (size_t)P.n + 2 * (size_t)P.ne + P.n_coef + P.nnz_lu + 64;
  CU(cudaMalloc(&stbuf.p, nd * sizeof(double)));
  CU(cudaMemsetAsync(stbuf.p, 0, nd * sizeof(double), c->stream));
  double *d = (double *)stbuf.p;
  TranState st;
  st.x = d; d += P.n;
  st.prev = d; d += P.n;
  st.guess = d; d += P.n;
  st.b = d; d += P.n;
  st.ca = d; d += P.n_coef;
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

namespace {

// Double-float direct engine launch for a group size G: instances per CTA (W) from the
// shared-memory footprint, the kernel instance and its residency.
using DfdKernel = void (*)(DevProg, KCfg, DfdLay, const double *, int, double, int, int, int, double *, int *, int *,
                           int, WaveTab, Probe, AdjFwd, Span, df *);
constexpr Span kWholeRun{1, 0, 0, nullptr};
// default options of the double-float engine (KRETS_DFD_OPTS overrides): trapezoidal
// capacitor history as companion currents (bit 2), measured 4 % faster on the RLC ladder;
// output conversion on the FP64 pipe in the direct-rhs step (bit 4; 4.81 -> 4.60 ms on
// 2048 instances x 200 steps of it: fewer issued instructions than integer widening)
constexpr int kDfdDefaultOpts = 4 | 16;
struct DfdLaunch {
  int G = 128, W = 1, per_sm = 0;
  bool lug = false;  // factors in global memory (k_tran_dfd<G, true>)
  size_t smem = 0;
  DfdKernel kd = nullptr;
  int slots() const { return W * per_sm * device_sm_count(); }
};

// Interleaved solves: factors in global memory and a program that has them (k_tran_dfd;
// one layout per group size).
bool dfd_interleaved(const DevProg &P, bool lug, int G) { return lug && P.il_ok; }

// interleaved layout of a group size (G = 64, 128, 32)
int il_layout(int G) { return G == 64 ? 0 : G == 128 ? 1 : 2; }

// The interleaved step with a direct right-hand side (dfd_steps_lean): a program that has
// one, TR with companion currents (opts bit 2) or BE; opts bit 3 turns it off.
bool dfd_lean_step(const DevProg &P, bool lug, int G, int method, int opts) {
  return dfd_interleaved(P, lug, G) && P.lean_ok && !(opts & 8) &&
         (method == KRETS_METHOD_BE || (method == KRETS_METHOD_TR && (opts & 4)));
}

// Shared-memory layout of one double-float instance (without the factors when lug: they
// are then in global memory); false when it does not fit a CTA.  G matters only with lug
// (the staged program then depends on it), method and opts only for the direct
// right-hand-side step (method < 0: never that step).
bool dfd_layout(const DevProg &P, DfdLay &DL, bool lug = false, int G = 64, int method = -1, int opts = 0) {
  size_t cur = 0;
  auto put = [&](int &off, size_t bytes) { off = (int)cur; cur = align16(cur + bytes); };
  const bool lean = method >= 0 && dfd_lean_step(P, lug, G, method, opts);
  DL.lean = lean ? 1 : 0;
  if (lug) DL.lu = 0;
  else put(DL.lu, 8 * (size_t)P.nnz_lu);
  if (lean) {  // two state buffers of n + 2 (ground zero, write-only slot)
    put(DL.x, 8 * ((size_t)P.n + 2));
    put(DL.cb, 8 * ((size_t)P.n + 2));
    put(DL.cdyn, 8 * (size_t)P.ndyn);
  } else {
    put(DL.x, 8 * (size_t)P.n);
    put(DL.cdyn, 8 * (size_t)P.ndyn);
    put(DL.cb, 8 * (size_t)P.ndyn);
  }
  put(DL.icap, 8 * (size_t)P.ncap);
  DL.coef64 = DL.x;  // set-up scratch over x / cdyn / cb / icap (+ padding if needed)
  if (cur - DL.x < 8 * (size_t)P.ne) cur = DL.x + align16(8 * (size_t)P.ne);
  put(DL.slot, 16);
  DL.bytes = (int)align16(cur);
  const int gi = il_layout(G);
  if (lean) {  // direct rhs records and unfed rows, output order, then the interleaved program
    DL.sprog_bytes = (int)(sizeof(int) * ((4 * (size_t)P.ndyn + P.n_zrow + 3) & ~(size_t)3) +
                           sizeof(int) * (((size_t)P.n + 3) & ~(size_t)3) +
                           sizeof(int) * (size_t)(P.ip_off[gi][3] - P.ip_off[gi][0]));
  } else if (dfd_interleaved(P, lug, G)) {  // rhs / gather / output sections, then the interleaved program
    DL.sprog_bytes = (int)(align16((size_t)(P.sp_off[5] - P.sp_off[7]) * sizeof(int)) +
                           align16((size_t)(P.ip_off[gi][3] - P.ip_off[gi][0]) * sizeof(int)));
  } else {
    DL.sprog_bytes = (int)align16((size_t)P.sp_off[5] * sizeof(int));
  }
  return (size_t)DL.bytes + DL.sprog_bytes <= max_smem_optin();
}

// Instances per CTA (W) from the shared-memory footprint, at most 896 threads per CTA (the
// kernel's launch bound) and 15 groups (named barriers 1..15) for G >= 64.
krets_status dfd_config(int G, bool lug, const DfdLay &DL, DfdLaunch &Lc) {
  Lc.G = G;
  Lc.lug = lug;
  const size_t cap = std::min<size_t>(896 / G, G >= 64 ? 15 : 28);
  Lc.W = (int)std::max<size_t>(1, std::min<size_t>(cap, (max_smem_optin() - DL.sprog_bytes) / DL.bytes));
  const char *wenv = getenv("KRETS_DFD_W");  // at most this many instances per CTA (tuning)
  if (wenv && atoi(wenv) > 0) Lc.W = std::min(Lc.W, atoi(wenv));
  Lc.smem = DL.sprog_bytes + (size_t)Lc.W * DL.bytes;
  if (lug) Lc.kd = G == 32 ? k_tran_dfd<32, true> : (G == 64 ? k_tran_dfd<64, true> : k_tran_dfd<128, true>);
  else Lc.kd = G == 32 ? k_tran_dfd<32> : (G == 64 ? k_tran_dfd<64> : k_tran_dfd<128>);
  CU(cudaFuncSetAttribute(Lc.kd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Lc.smem));
  CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&Lc.per_sm, Lc.kd, G * Lc.W, Lc.smem));
  if (Lc.per_sm < 1) return fail(KRETS_ERR_CUDA, "double-float engine does not fit on an SM");
  return KRETS_OK;
}

// Global-memory factors of every group of a launch (cached in the handle).
krets_status dfd_lu_buffer(krets_circuit *c, const DfdLaunch &Lc, int grid, const DevProg &P, df **out) {
  *out = nullptr;
  if (!Lc.lug) return KRETS_OK;
  // per group: the CSR factors, then (interleaved solves) their interleaved copy
  const size_t per = (size_t)P.nnz_lu + (dfd_interleaved(P, true, Lc.G) ? (size_t)P.il_slots[il_layout(Lc.G)] : 0);
  const size_t bytes = sizeof(df) * per * grid * Lc.W;
  krets_status s = c->ensure_lug(bytes);
  if (s != KRETS_OK) return s;
  *out = (df *)c->lug;
  return KRETS_OK;
}

// Autotuner of the double-float engine: the threads per instance (G = 128, 64, 32) and the
// place of the factors (shared memory, or global memory with more instances per SM) are
// chosen by timing one full wave of instances for up to 128 steps with each candidate, and
// ranking them by the time the whole batch would take (waves x wave time), once per
// sparsity signature (pattern hash, size, LU entries, method); the choice is cached for
// the process.  how = 1 measured now, 2 from the cache, 0 default (too few steps to time).
// A choice is kept as G | lug << 8.
std::mutex g_tune_mu;
std::map<std::string, int> g_tune;

std::string dfd_tune_key(const DevProgram *D, int method) {
  char key[96];
  snprintf(key, sizeof key, "%016llx/%d/%zu/%d", (unsigned long long)D->host.signature, D->host.n,
           D->host.lu_col.size(), method);
  return key;
}

krets_status dfd_pick(krets_circuit *c, const DevProgram *D, const double *dv, const double *dx, size_t stride,
                      int n_inst, double h, int n_steps, int method, int lag, int *queue, int opts, const WaveTab &wt,
                      const Probe &pr, int &G_out, bool &lug_out, int &how) {
  const std::string key = dfd_tune_key(D, method);
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(key);
    if (it != g_tune.end()) {
      G_out = it->second & 0xff;
      lug_out = (it->second >> 8) & 1;
      how = 2;
      return KRETS_OK;
    }
  }
  const DevProg &P = D->view;
  struct Cand { int G; bool lug; };
  const Cand cands[] = {{128, false}, {64, false}, {32, false}, {128, true}, {64, true}, {32, true}};
  std::vector<DfdLaunch> cfg;
  std::vector<DfdLay> lay;
  int trial_max = 1;
  for (const Cand &cd : cands) {
    DfdLay DL{};
    DfdLaunch Lc;
    if (!dfd_layout(P, DL, cd.lug, cd.G, method, opts) || dfd_config(cd.G, cd.lug, DL, Lc) != KRETS_OK) {
      cudaGetLastError();
      continue;
    }
    cfg.push_back(Lc);
    lay.push_back(DL);
    trial_max = std::max(trial_max, std::min(n_inst, Lc.slots()));
  }
  if (cfg.empty()) return fail(KRETS_ERR_INVALID_ARGUMENT, "double-float engine: no layout fits");
  // default (too few steps to time): the first candidate that fits
  G_out = cfg[0].G;
  lug_out = cfg[0].lug;
  how = 0;
  const int steps = std::min(n_steps, 128);
  if (steps < 16) return KRETS_OK;
  const int n = D->host.n;
  DevBuf tout, tst;
  const size_t row = sizeof(double) * (pr.n ? pr.n : n) * ((size_t)steps + 1);
  CU(cudaMalloc(&tout.p, row * trial_max));
  CU(cudaMalloc(&tst.p, sizeof(int) * trial_max));
  // the trial instances start from their operating points (row 0 of each waveform, or
  // the probe run's separate operating points)
  if (!pr.n && !pr.x0)
    CU(cudaMemcpy2DAsync(tout.p, row, dx, sizeof(double) * stride, sizeof(double) * n, trial_max,
                         cudaMemcpyDeviceToDevice, c->stream));
  double best = 0.0;
  for (size_t i = 0; i < cfg.size(); ++i) {
    const DfdLaunch &Lc = cfg[i];
    const int trial = std::max(1, std::min(n_inst, Lc.slots()));
    const int grid = std::max(1, std::min((trial + Lc.W - 1) / Lc.W, Lc.per_sm * device_sm_count()));
    df *lug = nullptr;
    krets_status s = dfd_lu_buffer(c, Lc, grid, P, &lug);
    if (s != KRETS_OK) return s;
    CU(cudaMemsetAsync(queue, 0, sizeof(int), c->stream));
    CU(cudaEventRecord(c->ev[2], c->stream));
    Lc.kd<<<grid, Lc.G * Lc.W, Lc.smem, c->stream>>>(D->view, c->cfg, lay[i], dv, trial, h, steps, method, lag,
                                                     (double *)tout.p, (int *)tst.p, queue, opts, wt, pr,
                                                     AdjFwd{nullptr, 1, 0, 0, nullptr}, kWholeRun, lug);
    g_launches++;
    CU(cudaGetLastError());
    CU(cudaEventRecord(c->ev[3], c->stream));
    CU(cudaEventSynchronize(c->ev[3]));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c->ev[2], c->ev[3]);
    const double waves = std::ceil((double)n_inst / std::max(1, Lc.slots()));
    const double predicted = waves * ms;  // the whole batch, for these steps
    if (ms > 0.f && (best == 0.0 || predicted < best)) {
      best = predicted;
      G_out = Lc.G;
      lug_out = Lc.lug;
    }
  }
  how = 1;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tune[key] = G_out | (lug_out ? 1 << 8 : 0);
  return KRETS_OK;
}

// Group size of the double-float engine without a trial run: KRETS_GROUP, else the
// autotuner's cached choice for this sparsity signature, else the default 128.  (The
// place of the factors does not change the arithmetic, only the group size does.)
int dfd_cached_group(const DevProgram *D, int method, int &how) {
  const char *genv = getenv("KRETS_GROUP");
  how = 0;
  if (genv) {
    const int G = atoi(genv);
    return (G == 32 || G == 64 || G == 128) ? G : 128;
  }
  const std::string key = dfd_tune_key(D, method);
  std::lock_guard<std::mutex> lk(g_tune_mu);
  auto it = g_tune.find(key);
  if (it == g_tune.end()) return 128;
  how = 2;
  return it->second & 0xff;
}

// Shared-memory layout of one warp of the warp engine (k_tran_warp, k_tran_warp_df);
// returns the bytes per warp.
size_t warp_layout(const DevProg &P, bool mixed, WarpLay &WL) {
  size_t cur = 0;
  auto put = [&](int &off, size_t bytes) { off = (int)cur; cur = align16(cur + bytes); };
  put(WL.lu, (mixed ? 4 : 8) * (size_t)P.nnz_lu);
  put(WL.coef, 8 * (size_t)P.ne);
  put(WL.x, 8 * (size_t)P.n);
  put(WL.b, 8 * (size_t)P.n);
  put(WL.w, mixed ? 4 * (size_t)P.n : 16);
  put(WL.cb, 8 * (size_t)P.ndyn);
  put(WL.icap, 8 * (size_t)P.ncap);
  put(WL.prev, P.nonlinear ? 8 * (size_t)P.n : 0);
  put(WL.guess, P.nonlinear ? 8 * (size_t)P.n : 0);
  WL.bytes = (int)align16(cur);
  WL.sprog_bytes = (int)align16((size_t)P.sp_off[11] * sizeof(int));
  return (size_t)WL.bytes;
}

// Warps per CTA of the warp engine (KRETS_SMEM_BUDGET and KRETS_WARPS_PER_CTA override).
int warp_engine_width(const WarpLay &WL, size_t per_warp) {
  const char *bud = getenv("KRETS_SMEM_BUDGET");
  size_t budget = bud ? (size_t)atol(bud) : max_smem_optin();
  budget = std::min(budget, max_smem_optin());
  int W = (int)std::max<size_t>(1, std::min<size_t>(8, (budget - WL.sprog_bytes) / per_warp));
  const char *wenv = getenv("KRETS_WARPS_PER_CTA");
  if (wenv) W = std::max(1, std::min(8, atoi(wenv)));
  while (W > 1 && WL.sprog_bytes + (size_t)W * per_warp > max_smem_optin()) --W;
  return W;
}

// PULSE / SIN sources of a transient program that the double-float engine tabulates per
// step: wrow[d] = table row of rhs element d (or -1), wsrc = their element indices.
void wave_sources(const krets_circuit *c, const Program &H, int ndyn, std::vector<int> &wrow, std::vector<int> &wsrc) {
  wrow.assign(ndyn, -1);
  wsrc.clear();
  for (int d = 0; d < ndyn; ++d) {
    const krets_element &E = c->el[H.dyn_e[d]];
    if (E.kind == KRETS_ELEM_V && E.wave != KRETS_WAVE_NONE) {
      wrow[d] = (int)wsrc.size();
      wsrc.push_back(H.dyn_e[d]);
    }
  }
}

}  // namespace

// Batched transient; with probes (n_probe > 0) only those unknowns are written each step
// (double-float engine only): x_out[n_inst][n_steps+1][n_probe].
static krets_status batch_tran_impl(krets_circuit *c, int32_t n_inst, const double *values, double h,
                                    int32_t n_steps, int32_t method, int32_t source_lag, int32_t precision,
                                    double *x_out, int32_t *inst_status, const int32_t *probe, int32_t n_probe) {
  if (!c || !x_out || n_inst <= 0 || n_steps < 0 || !(h > 0)) return fail(KRETS_ERR_INVALID_ARGUMENT, "invalid arguments");
  DevProgram *Ddc, *Dtr;
  krets_status s = get_program(c, MODE_DC, 0, 0, 0, &Ddc);
  if (s != KRETS_OK) return s;
  s = get_program(c, MODE_TRAN, method, h, 0, &Dtr);
  if (s != KRETS_OK) return s;
  const DevProg &P = Dtr->view;
  const char *eng = getenv("KRETS_ENGINE");
  const bool block_forced = eng && strcmp(eng, "block") == 0;
  // double-float direct: one instance per group of G threads (default 128); it stages only
  // the step-program words before the residual operators, so it fits where the warp
  // engine may not
  const char *oenv = getenv("KRETS_DFD_OPTS");
  const int opts = oenv ? atoi(oenv) : kDfdDefaultOpts;
  DfdLay DL{}, DLg{};
  const bool dfd_smem = dfd_layout(P, DL), dfd_glob = dfd_layout(P, DLg, true, 64, method, opts);
  const bool use_dfd = precision == KRETS_PREC_DF && !P.nonlinear && P.sprog_ok && !block_forced && (dfd_smem || dfd_glob);
  // Host output of the double-float engine is staged: the transient runs as spans of
  // steps, each written to a device staging buffer and copied into the caller's rows by
  // one strided copy on a second stream while the next span runs.  That is the path for
  // pinned host buffers, and for any host buffer where the GPU cannot write host memory
  // in place; pageable buffers on a GPU that shares the host's page tables are written in
  // place by the kernel, which measured faster for them.  KRETS_HOST_OUT=inplace|staged
  // forces either.
  const char *hout = getenv("KRETS_HOST_OUT");
  const size_t out_bytes = sizeof(double) * (size_t)(n_probe > 0 ? n_probe : c->n) * ((size_t)n_steps + 1) * n_inst;
  const bool host_out = !is_device_ptr(x_out);
  bool want_staged = host_out && (!direct_host_access() || is_pinned_host(x_out, out_bytes));
  if (hout) want_staged = host_out && strcmp(hout, "staged") == 0;
  const bool staged = want_staged && use_dfd && n_probe <= 0 && n_steps >= 2 &&
                      sizeof(double) * (size_t)c->n * ((size_t)n_steps + 1) < ((size_t)1 << 31);  // copy pitch
  CU(cudaEventRecord(c->ev[0], c->stream));
  const int n_out = n_probe > 0 ? n_probe : c->n;
  size_t stride = (size_t)n_out * ((size_t)n_steps + 1);
  DevBuf tv, tx, ts, tfb, twave, top, tprobe, tstate;
  void *dv, *dx = nullptr;
  if (staged && values && !is_device_ptr(values)) {  // read once per span: keep a device copy
    CU(cudaMalloc(&tv.p, sizeof(double) * c->ne * (size_t)n_inst));
    CU(cudaMemcpyAsync(tv.p, values, sizeof(double) * c->ne * (size_t)n_inst, cudaMemcpyHostToDevice, c->stream));
    dv = tv.p;
  } else {
    s = dev_view(values, sizeof(double) * c->ne * (size_t)n_inst, true, c->stream, tv, &dv);
    if (s) return s;
  }
  if (!staged) {
    s = dev_view(x_out, sizeof(double) * stride * n_inst, false, c->stream, tx, &dx);
    if (s) return s;
  }
  CU(cudaMalloc(&ts.p, sizeof(int) * 2 * (size_t)n_inst));
  int *d_st = (int *)ts.p, *d_opst = d_st + n_inst;
  CU(cudaMemsetAsync(ts.p, 0, sizeof(int) * 2 * (size_t)n_inst, c->stream));
  Probe pr{nullptr, 0, nullptr};
  if (staged) {
    // operating points in a separate [n_inst][n] buffer (copied to row 0 of each instance)
    CU(cudaMalloc(&top.p, sizeof(double) * c->n * (size_t)n_inst));
    pr = Probe{nullptr, 0, (const double *)top.p};
    s = run_op(c, Ddc, n_inst, (const double *)dv, (double *)top.p, c->n, d_opst, nullptr, 128);
  } else if (n_probe > 0) {
    // operating points in a separate [n_inst][n] buffer; the probe list on the device
    CU(cudaMalloc(&top.p, sizeof(double) * c->n * (size_t)n_inst));
    void *dp;
    s = dev_view(probe, sizeof(int32_t) * n_probe, true, c->stream, tprobe, &dp);
    if (s) return s;
    pr = Probe{(const int *)dp, n_probe, (const double *)top.p};
    s = run_op(c, Ddc, n_inst, (const double *)dv, (double *)top.p, c->n, d_opst, nullptr, 128);
  } else {
    s = run_op(c, Ddc, n_inst, (const double *)dv, (double *)dx, stride, d_opst, nullptr, 128);
  }
  if (s) return s;
  const bool dfd = precision == KRETS_PREC_DF;
  bool mixed = precision == KRETS_PREC_MIXED;
  if (dfd && P.nonlinear) mixed = true;  // nonlinear circuits: refactor per Newton iteration (FP32 + refinement)
  int *queue = c->d_small + 8;
  int *d_fallbacks = c->d_small + 12;
  CU(cudaMemsetAsync(c->d_small + 8, 0, 8 * sizeof(int), c->stream));
  CU(cudaMemsetAsync(c->d_hist, 0, 8 * sizeof(unsigned long long), c->stream));
  bool warp_engine = !block_forced;
  WarpLay WL{};
  size_t per_warp = 0;
  if (warp_engine) {
    per_warp = warp_layout(P, mixed, WL);
    if (!P.sprog_ok || per_warp + WL.sprog_bytes > max_smem_optin()) warp_engine = false;
  }
  double *fb = nullptr;
  if (n_probe > 0 && !use_dfd)
    return fail(KRETS_ERR_INVALID_ARGUMENT,
                "probe outputs need the double-float engine (precision 2, a linear circuit that fits)");
  if (use_dfd) {
    // PULSE / SIN sources tabulated per step (their parameters are not per-instance values)
    std::vector<int> wrow, wsrc;
    wave_sources(c, Dtr->host, P.ndyn, wrow, wsrc);
    WaveTab wt{nullptr, nullptr, n_steps + 1};
    if (!wsrc.empty()) {
      const size_t tab_bytes = sizeof(double) * wsrc.size() * (size_t)(n_steps + 1);
      CU(cudaMalloc(&twave.p, tab_bytes + sizeof(int) * (wrow.size() + wsrc.size())));
      int *d_wrow = (int *)((char *)twave.p + tab_bytes), *d_wsrc = d_wrow + wrow.size();
      CU(cudaMemcpyAsync(d_wrow, wrow.data(), sizeof(int) * wrow.size(), cudaMemcpyHostToDevice, c->stream));
      CU(cudaMemcpyAsync(d_wsrc, wsrc.data(), sizeof(int) * wsrc.size(), cudaMemcpyHostToDevice, c->stream));
      k_wave_table<<<256, 256, 0, c->stream>>>(c->d_el, d_wsrc, (int)wsrc.size(), h, n_steps, source_lag,
                                              (double *)twave.p);
      g_launches++;
      CU(cudaGetLastError());
      wt.tab = (const double *)twave.p;
      wt.row = d_wrow;
    }
    // group size and place of the factors: KRETS_GROUP / KRETS_DFD_LU (smem | global),
    // else the autotuner
    const char *genv = getenv("KRETS_GROUP"), *lenv = getenv("KRETS_DFD_LU");
    int G = 128, how = 0;
    bool lug = !dfd_smem;
    if (genv || lenv) {
      if (genv) G = atoi(genv);
      if (G != 32 && G != 64 && G != 128) G = 128;
      if (lenv) lug = strcmp(lenv, "global") == 0 || !dfd_smem;
    } else {
      s = dfd_pick(c, Dtr, (const double *)dv, (const double *)dx, stride, n_inst, h, n_steps, method, source_lag,
                   queue, opts, wt, pr, G, lug, how);
      if (s != KRETS_OK) return s;
    }
    if (lug && !dfd_layout(P, DL, true, G, method, opts))
      return fail(KRETS_ERR_INVALID_ARGUMENT, "double-float layout does not fit");
    DfdLaunch Lc;
    s = dfd_config(G, lug, DL, Lc);
    if (s != KRETS_OK) return s;
    const int W = Lc.W;
    int grid = std::max(1, std::min((n_inst + W - 1) / W, Lc.per_sm * device_sm_count()));
    df *lu_glob = nullptr;
    s = dfd_lu_buffer(c, Lc, grid, P, &lu_glob);
    if (s != KRETS_OK) return s;
    c->warps_per_cta = W * G / 32;
    c->grid = grid;
    c->launch_info[0] = G;
    c->launch_info[1] = W;
    c->launch_info[2] = grid;
    c->launch_info[3] = how;
    c->launch_info[4] = lug ? 1 : 0;
    if (!staged) {
      CU(cudaMemsetAsync(queue, 0, sizeof(int), c->stream));
      CU(cudaEventRecord(c->ev[2], c->stream));
      Lc.kd<<<grid, G * W, Lc.smem, c->stream>>>(P, c->cfg, DL, (const double *)dv, n_inst, h, n_steps, method,
                                                 source_lag, (double *)dx, d_st, queue, opts, wt, pr,
                                                 AdjFwd{nullptr, 1, 0, 0, nullptr}, kWholeRun, lu_glob);
    } else {
      // spans of R steps; two staging buffers of n_inst x R rows (KRETS_STAGE_MB each,
      // default 2048), at least 8 spans
      const size_t row_bytes = sizeof(double) * c->n * (size_t)n_inst;
      const char *smb = getenv("KRETS_STAGE_MB");
      const size_t budget = (smb ? (size_t)std::max(1, atoi(smb)) : 2048) << 20;
      const int R = (int)std::max<size_t>(1, std::min<size_t>((n_steps + 7) / 8, budget / row_bytes));
      const int nspan = (n_steps + R - 1) / R;
      s = c->ensure_stage(2 * (size_t)R * row_bytes);
      if (s != KRETS_OK) return s;
      double *stage[2] = {(double *)c->stage, (double *)c->stage + (size_t)R * c->n * n_inst};
      CU(cudaMalloc(&tstate.p, sizeof(df) * ((size_t)P.n + P.ncap) * n_inst));
      cudaEvent_t *kdone = c->sev, *copied = c->sev + 2, op_done = c->sev[4];
      const size_t pitch = sizeof(double) * stride;
      auto launch = [&](int j) -> krets_status {
        const int s0 = j * R + 1, s1 = std::min(n_steps, (j + 1) * R);
        if (j >= 2) CU(cudaStreamWaitEvent(c->stream, copied[j & 1], 0));  // its buffer has been copied out
        CU(cudaMemsetAsync(queue, 0, sizeof(int), c->stream));
        Lc.kd<<<grid, G * W, Lc.smem, c->stream>>>(P, c->cfg, DL, (const double *)dv, n_inst, h, s1, method,
                                                   source_lag, stage[j & 1], d_st, queue, opts, wt, pr,
                                                   AdjFwd{nullptr, 1, 0, 0, nullptr},
                                                   Span{s0, s0, (long long)R * c->n, (df *)tstate.p}, lu_glob);
        g_launches++;
        CU(cudaGetLastError());
        CU(cudaEventRecord(kdone[j & 1], c->stream));
        return KRETS_OK;
      };
      auto copy_out = [&](int j) -> krets_status {
        const int s0 = j * R + 1, s1 = std::min(n_steps, (j + 1) * R);
        CU(cudaStreamWaitEvent(c->copy_stream, kdone[j & 1], 0));
        CU(cudaMemcpy2DAsync(x_out + (size_t)s0 * c->n, pitch, stage[j & 1], sizeof(double) * R * c->n,
                             sizeof(double) * (size_t)(s1 - s0 + 1) * c->n, n_inst, cudaMemcpyDeviceToHost,
                             c->copy_stream));
        CU(cudaEventRecord(copied[j & 1], c->copy_stream));
        return KRETS_OK;
      };
      CU(cudaEventRecord(c->ev[2], c->stream));
      // each span's copy is issued after the next span's launch, so the copies overlap
      // the kernels even where a copy into pageable memory returns only when it is done
      s = launch(0);
      if (s != KRETS_OK) return s;
      CU(cudaEventRecord(op_done, c->stream));
      CU(cudaStreamWaitEvent(c->copy_stream, op_done, 0));
      CU(cudaMemcpy2DAsync(x_out, pitch, top.p, sizeof(double) * c->n, sizeof(double) * c->n, n_inst,
                           cudaMemcpyDeviceToHost, c->copy_stream));  // row 0: the operating points
      for (int j = 0; j < nspan; ++j) {
        if (j + 1 < nspan) {
          s = launch(j + 1);
          if (s != KRETS_OK) return s;
        }
        s = copy_out(j);
        if (s != KRETS_OK) return s;
      }
      CU(cudaEventRecord(c->ev[3], c->stream));
      CU(cudaEventRecord(op_done, c->copy_stream));
      CU(cudaStreamWaitEvent(c->stream, op_done, 0));  // every copy is done before the call returns
    }
  } else if (warp_engine) {
    const int W = warp_engine_width(WL, per_warp);
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
  if (!staged) {
    g_launches++;
    CU(cudaGetLastError());
    CU(cudaEventRecord(c->ev[3], c->stream));
  }
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

krets_status krets_batch_tran(krets_circuit *c, int32_t n_inst, const double *values, double h, int32_t n_steps,
                              int32_t method, int32_t source_lag, int32_t precision, double *x_out,
                              int32_t *inst_status) {
  return batch_tran_impl(c, n_inst, values, h, n_steps, method, source_lag, precision, x_out, inst_status, nullptr, 0);
}

krets_status krets_batch_tran_probe(krets_circuit *c, int32_t n_inst, const double *values, double h, int32_t n_steps,
                                    int32_t method, int32_t source_lag, int32_t n_probe, const int32_t *probe,
                                    double *x_out, int32_t *inst_status) {
  if (!c || !probe || n_probe <= 0) return fail(KRETS_ERR_INVALID_ARGUMENT, "invalid probe list");
  // the kernel indexes shared memory with these: check every index on the host
  std::vector<int32_t> hp(n_probe);
  if (is_device_ptr(probe)) CU(cudaMemcpy(hp.data(), probe, sizeof(int32_t) * n_probe, cudaMemcpyDeviceToHost));
  else memcpy(hp.data(), probe, sizeof(int32_t) * n_probe);
  for (int32_t v : hp)
    if (v < 0 || v >= c->n) return fail(KRETS_ERR_INVALID_ARGUMENT, "probe index out of range");
  return batch_tran_impl(c, n_inst, values, h, n_steps, method, source_lag, KRETS_PREC_DF, x_out, inst_status, probe,
                         n_probe);
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
  std::vector<int> adj(4 * (size_t)P.ne, -1), ccp(P.n + 1, 0), cco, dyn_of(P.ne, -1);
  std::vector<std::vector<int>> cols(P.n);
  for (size_t d = 0; d < H.dyn_e.size(); ++d) dyn_of[H.dyn_e[d]] = (int)d;
  for (int e = 0; e < P.ne; ++e) {
    const krets_element &E = c->el[e];
    if ((E.kind == KRETS_ELEM_R || E.kind == KRETS_ELEM_C) && (E.flags & KRETS_FLAG_G2))
      return fail(KRETS_ERR_NOT_IMPLEMENTED, "adjoint sensitivities of group-2 resistor/capacitor stamps");
    // kind, and for sources the rhs-element index (their per-step values come from it)
    const bool src = (E.kind == KRETS_ELEM_V || E.kind == KRETS_ELEM_I) && dyn_of[e] >= 0;
    adj[4 * e] = E.kind | (src ? (dyn_of[e] + 1) << 8 : 0);
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
  // The forward pass runs on the double-float transient engine when the instance fits it
  // (several instances per SM, checkpoints per instance), then the reverse sweep runs here
  // (mode 2); otherwise both run in this kernel (checkpoints per CTA).
  // KRETS_ADJ_SINGLE=1 forces the single-kernel form.
  DfdLay DL{};
  const char *single = getenv("KRETS_ADJ_SINGLE");
  const bool split = dfd_layout(P, DL) && !(single && single[0] == '1');
  CU(cudaMalloc(&tck.p, sizeof(df) * (size_t)(split ? n_inst : grid) * J * ((size_t)P.n + P.ncap)));
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
  // PULSE / SIN sources tabulated per step (sources at t_n, no lag)
  DevBuf twave;
  WaveTab wt{nullptr, nullptr, n_steps + 1};
  {
    std::vector<int> wrow(P.ndyn, -1), wsrc;
    for (int d = 0; d < P.ndyn; ++d) {
      const krets_element &E = c->el[H.dyn_e[d]];
      if (E.kind == KRETS_ELEM_V && E.wave != KRETS_WAVE_NONE) {
        wrow[d] = (int)wsrc.size();
        wsrc.push_back(H.dyn_e[d]);
      }
    }
    if (!wsrc.empty()) {
      const size_t tab_bytes = sizeof(double) * wsrc.size() * (size_t)(n_steps + 1);
      CU(cudaMalloc(&twave.p, tab_bytes + sizeof(int) * (wrow.size() + wsrc.size())));
      int *d_wrow = (int *)((char *)twave.p + tab_bytes), *d_wsrc = d_wrow + wrow.size();
      CU(cudaMemcpyAsync(d_wrow, wrow.data(), sizeof(int) * wrow.size(), cudaMemcpyHostToDevice, c->stream));
      CU(cudaMemcpyAsync(d_wsrc, wsrc.data(), sizeof(int) * wsrc.size(), cudaMemcpyHostToDevice, c->stream));
      k_wave_table<<<256, 256, 0, c->stream>>>(c->d_el, d_wsrc, (int)wsrc.size(), h, n_steps, 0, (double *)twave.p);
      g_launches++;
      CU(cudaGetLastError());
      wt.tab = (const double *)twave.p;
      wt.row = d_wrow;
    }
  }
  DevBuf tstf;
  CU(cudaMalloc(&tstf.p, sizeof(int) * n_inst));
  CU(cudaMemsetAsync(tstf.p, 0, sizeof(int) * n_inst, c->stream));
  // The forward pass takes the transient engine's configuration for this circuit (group
  // size and place of the factors from the autotuner, whose trial runs start from the
  // zero operating points in top; the direct right-hand-side step when it applies, whose
  // checkpoints then hold the capacitors' companion values: ck_cb).
  DfdLaunch Lf;
  DfdLay DLf{};
  df *lu_glob = nullptr;
  int fgrid = 1, fopts = 0, ck_cb = 0;
  if (split) {
    const char *oenv = getenv("KRETS_DFD_OPTS");
    fopts = oenv ? atoi(oenv) : kDfdDefaultOpts;
    int G = 128, how = 0;
    bool lug = false;
    s = dfd_pick(c, Dtr, (const double *)dv, nullptr, 0, n_inst, h, n_steps, method, 0, queue, fopts, wt,
                 Probe{nullptr, 0, (const double *)top.p}, G, lug, how);
    if (s != KRETS_OK) return s;
    if (!dfd_layout(P, DLf, lug, G, method, fopts)) {
      G = 128;
      lug = false;
      if (!dfd_layout(P, DLf, false, G, method, fopts)) return fail(KRETS_ERR_INVALID_ARGUMENT, "double-float layout does not fit");
    }
    s = dfd_config(G, lug, DLf, Lf);
    if (s != KRETS_OK) return s;
    fgrid = std::max(1, std::min((n_inst + Lf.W - 1) / Lf.W, Lf.per_sm * device_sm_count()));
    s = dfd_lu_buffer(c, Lf, fgrid, P, &lu_glob);
    if (s != KRETS_OK) return s;
    ck_cb = DLf.lean && method == KRETS_METHOD_TR;
    CU(cudaMemsetAsync(queue, 0, sizeof(int), c->stream));
  }
  CU(cudaEventRecord(c->ev[2], c->stream));
  if (split) {
    const AdjFwd af{(df *)tck.p, K, P.n + P.ncap, H.qinv[out_unknown], (double *)d_loss};
    Lf.kd<<<fgrid, Lf.G * Lf.W, Lf.smem, c->stream>>>(P, c->cfg, DLf, (const double *)dv, n_inst, h, n_steps,
                                                      method, 0, nullptr, (int *)tstf.p, queue, fopts, wt,
                                                      Probe{nullptr, 0, nullptr}, af, kWholeRun, lu_glob);
    g_launches++;
    CU(cudaGetLastError());
    CU(cudaMemsetAsync(queue, 0, sizeof(int), c->stream));
  }
  if (!split || gradient) {
    ka<<<grid, kAdjThreads, smem, c->stream>>>(P, AL, (const double *)dv, n_inst, h, n_steps, method, K,
                                               H.qinv[out_unknown], (const int4 *)d_adj, d_ccp, d_cco, (df *)tck.p,
                                               (df *)tseg.p, d_hist, (double *)d_loss, (double *)d_grad,
                                               (int *)tst.p, queue, split ? 2 : (gradient ? 1 : 0), wt, ck_cb);
    g_launches++;
    CU(cudaGetLastError());
  }
  CU(cudaEventRecord(c->ev[3], c->stream));
  if (dl_loss.p) CU(cudaMemcpyAsync(loss_out, d_loss, sizeof(double) * n_inst, cudaMemcpyDeviceToHost, c->stream));
  if (dl_grad.p)
    CU(cudaMemcpyAsync(grad_out, d_grad, sizeof(double) * (size_t)n_inst * c->ne, cudaMemcpyDeviceToHost, c->stream));
  std::vector<int> st(n_inst), stf(n_inst);
  CU(cudaMemcpyAsync(st.data(), tst.p, sizeof(int) * n_inst, cudaMemcpyDeviceToHost, c->stream));
  CU(cudaMemcpyAsync(stf.data(), tstf.p, sizeof(int) * n_inst, cudaMemcpyDeviceToHost, c->stream));
  CU(cudaEventRecord(c->ev[1], c->stream));
  CU(cudaStreamSynchronize(c->stream));
  cudaEventElapsedTime(&c->kernel_ms, c->ev[2], c->ev[3]);
  cudaEventElapsedTime(&c->call_ms, c->ev[0], c->ev[1]);
  c->warps_per_cta = kAdjThreads / 32;
  c->grid = grid;
  int any = 0;
  for (int i = 0; i < n_inst; ++i) any |= st[i] | stf[i];
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

krets_status krets_last_launch(const krets_circuit *c, int32_t *info, int32_t cap) {
  if (!c || !info) return fail(KRETS_ERR_INVALID_ARGUMENT, "invalid arguments to krets_last_launch");
  for (int i = 0; i < cap && i < 5; ++i) info[i] = c->launch_info[i];
  return KRETS_OK;
}

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

krets_status krets_host_register(void *ptr, size_t bytes) {
  if (!ptr || !bytes) return fail(KRETS_ERR_INVALID_ARGUMENT, "null or empty host buffer");
  CU(cudaHostRegister(ptr, bytes, cudaHostRegisterDefault));
  return KRETS_OK;
}

krets_status krets_host_unregister(void *ptr) {
  if (!ptr) return fail(KRETS_ERR_INVALID_ARGUMENT, "null host buffer");
  CU(cudaHostUnregister(ptr));
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
// For each precision it makes the same engine choice, with the same kernels, group size,
// tolerances and launch parameters, as krets_batch_tran with device-resident buffers, so
// the results are identical; what that call would allocate (status words, the work-queue
// counter, the source-waveform table, FP64 fallback factors) comes from g_noalloc_scratch.
// Circuits that krets_batch_tran runs with global-memory workspaces are rejected.
krets_status krets_batch_tran_noalloc(krets_circuit *c, int32_t n_inst, const double *d_values, double h,
                                      int32_t n_steps, int32_t method, int32_t source_lag, int32_t precision,
                                      double *d_x_out, int32_t *d_inst_status) {
  if (!c || n_inst <= 0 || n_steps < 0 || !(h > 0) || !d_x_out || !d_inst_status)
    return fail(KRETS_ERR_INVALID_ARGUMENT, "invalid arguments to krets_batch_tran_noalloc");
  if (precision != KRETS_PREC_FP64 && precision != KRETS_PREC_MIXED && precision != KRETS_PREC_DF)
    return fail(KRETS_ERR_INVALID_ARGUMENT, "krets_batch_tran_noalloc: unknown precision");
  if ((d_values && !is_device_ptr(d_values)) || !is_device_ptr(d_x_out) || !is_device_ptr(d_inst_status))
    return fail(KRETS_ERR_INVALID_ARGUMENT, "krets_batch_tran_noalloc needs device pointers for values, "
                                            "x_out and inst_status");
  DevProgram *Ddc = find_program(c, MODE_DC, 0, 0, 0);
  DevProgram *Dtr = find_program(c, MODE_TRAN, method, h, 0);
  if (!Ddc || !Dtr)
    return fail(KRETS_ERR_INVALID_ARGUMENT, "krets_batch_tran_noalloc: the circuit has no compiled program for this "
                                            "time step and method; run krets_batch_tran once with them first");
  const DevProg &P = Dtr->view;
  // operating point: its per-CTA workspace must fit in shared memory (no global workspace)
  if (layout_op(Ddc->view).bytes > max_smem_optin())
    return fail(KRETS_ERR_INVALID_ARGUMENT, "krets_batch_tran_noalloc: circuit too large for the shared-memory "
                                            "operating-point kernel");
  // engine choice, as in batch_tran_impl
  const bool dfd = precision == KRETS_PREC_DF;
  bool mixed = precision == KRETS_PREC_MIXED;
  if (dfd && P.nonlinear) mixed = true;
  const char *eng = getenv("KRETS_ENGINE");
  const bool block_forced = eng && strcmp(eng, "block") == 0;
  DfdLay DL{};
  const bool use_dfd = dfd && !P.nonlinear && P.sprog_ok && !block_forced && dfd_layout(P, DL);
  if (dfd && !P.nonlinear && P.sprog_ok && !block_forced && !use_dfd)
    // krets_batch_tran runs such a circuit with its factors in global memory it allocates
    return fail(KRETS_ERR_INVALID_ARGUMENT, "krets_batch_tran_noalloc: circuit too large for the shared-memory "
                                            "double-float engine");
  WarpLay WL{};
  const size_t per_warp = warp_layout(P, mixed, WL);
  const bool warp_engine = !use_dfd && !block_forced && P.sprog_ok && per_warp + WL.sprog_bytes <= max_smem_optin();
  if (!use_dfd && !warp_engine)
    return fail(KRETS_ERR_INVALID_ARGUMENT, "krets_batch_tran_noalloc: circuit too large for the shared-memory "
                                            "transient engines");
  const char *dfenv = getenv("KRETS_DF");
  const bool use_df = warp_engine && mixed && !P.nonlinear && !(dfenv && dfenv[0] == '0');
  const bool need_fb = warp_engine && mixed && !use_df;  // k_tran_warp<1>: FP64 fallback factors
  // scratch layout: [0,64) counters and summary words, [64,128) refinement histogram,
  // [256, ..) operating-point status per instance, then the waveform table (double-float
  // engine with PULSE / SIN sources), then the FP64 fallback factors of every warp slot
  std::vector<int> wrow, wsrc;
  if (use_dfd) wave_sources(c, Dtr->host, P.ndyn, wrow, wsrc);
  const size_t op_off = 256;
  const size_t tab_off = align16(op_off + sizeof(int) * (size_t)n_inst);
  const size_t tab_bytes = wsrc.empty() ? 0 : sizeof(double) * wsrc.size() * ((size_t)n_steps + 1);
  const size_t wrow_off = tab_off + tab_bytes;
  const size_t wsrc_off = wrow_off + sizeof(int) * wrow.size();
  const size_t lu_off = align16(wsrc.empty() ? tab_off : wsrc_off + sizeof(int) * wsrc.size());
  if (lu_off > KRETS_NOALLOC_SCRATCH_BYTES)
    return fail(KRETS_ERR_INVALID_ARGUMENT, "krets_batch_tran_noalloc: instances x steps exceed the 16 MiB scratch");
  void *scr = nullptr;
  krets_status s = noalloc_scratch_address(&scr);
  if (s) return s;
  char *base = (char *)scr;
  int *queue = (int *)(base + 0);
  int *fallbacks = (int *)(base + 4);
  int *any_op = (int *)(base + 8);
  int *any_tran = (int *)(base + 12);
  unsigned long long *hist = (unsigned long long *)(base + 64);
  int *op_status = (int *)(base + op_off);
  CU(cudaEventRecord(c->ev[0], c->stream));
  // everything that must start at zero: counters, summary words, histogram, statuses
  CU(cudaMemsetAsync(base, 0, 256, c->stream));
  CU(cudaMemsetAsync(op_status, 0, sizeof(int) * (size_t)n_inst, c->stream));
  CU(cudaMemsetAsync(d_inst_status, 0, sizeof(int) * (size_t)n_inst, c->stream));
  const size_t stride = (size_t)c->n * ((size_t)n_steps + 1);
  // the operating-point workspace fits in shared memory, so run_op allocates nothing
  s = run_op(c, Ddc, n_inst, d_values, d_x_out, stride, op_status, nullptr, 128);
  if (s) return s;
  if (use_dfd) {
    WaveTab wt{nullptr, nullptr, n_steps + 1};
    if (!wsrc.empty()) {
      int *d_wrow = (int *)(base + wrow_off), *d_wsrc = (int *)(base + wsrc_off);
      CU(cudaMemcpyAsync(d_wrow, wrow.data(), sizeof(int) * wrow.size(), cudaMemcpyHostToDevice, c->stream));
      CU(cudaMemcpyAsync(d_wsrc, wsrc.data(), sizeof(int) * wsrc.size(), cudaMemcpyHostToDevice, c->stream));
      k_wave_table<<<256, 256, 0, c->stream>>>(c->d_el, d_wsrc, (int)wsrc.size(), h, n_steps, source_lag,
                                              (double *)(base + tab_off));
      g_launches++;
      CU(cudaGetLastError());
      wt.tab = (const double *)(base + tab_off);
      wt.row = d_wrow;
    }
    const char *oenv = getenv("KRETS_DFD_OPTS");
    const int opts = oenv ? atoi(oenv) : kDfdDefaultOpts;
    int how = 0;
    const int G = dfd_cached_group(Dtr, method, how);  // never a trial run: it would allocate
    DfdLaunch Lc;
    s = dfd_config(G, false, DL, Lc);
    if (s != KRETS_OK) return s;
    const int grid = std::max(1, std::min((n_inst + Lc.W - 1) / Lc.W, Lc.per_sm * device_sm_count()));
    c->warps_per_cta = Lc.W * G / 32;
    c->grid = grid;
    c->launch_info[0] = G;
    c->launch_info[1] = Lc.W;
    c->launch_info[2] = grid;
    c->launch_info[3] = how;
    c->launch_info[4] = 0;
    CU(cudaEventRecord(c->ev[2], c->stream));
    Lc.kd<<<grid, G * Lc.W, Lc.smem, c->stream>>>(P, c->cfg, DL, d_values, n_inst, h, n_steps, method, source_lag,
                                                  d_x_out, d_inst_status, queue, opts, wt, Probe{nullptr, 0, nullptr},
                                                  AdjFwd{nullptr, 1, 0, 0, nullptr}, kWholeRun, nullptr);
  } else {
    const int W = warp_engine_width(WL, per_warp);
    const size_t smem = WL.sprog_bytes + (size_t)W * per_warp;
    auto kern = mixed ? k_tran_warp<1> : k_tran_warp<0>;
    int per_sm = 0;
    if (use_df) {
      CU(cudaFuncSetAttribute(k_tran_warp_df, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tran_warp_df, 32 * W, smem));
    } else {
      CU(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
      CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32 * W, smem));
    }
    if (per_sm < 1) return fail(KRETS_ERR_CUDA, "warp engine does not fit on an SM");
    int grid = std::max(1, std::min((n_inst + W - 1) / W, per_sm * device_sm_count()));
    double *fb = nullptr;
    if (need_fb) {
      // one factor slot per warp of the grid; fewer slots only mean fewer resident CTAs
      // (each instance's arithmetic does not depend on the grid)
      const size_t lu_slot = sizeof(double) * (size_t)P.nnz_lu;
      const size_t slots = lu_off < KRETS_NOALLOC_SCRATCH_BYTES ? (KRETS_NOALLOC_SCRATCH_BYTES - lu_off) / lu_slot : 0;
      if (slots < (size_t)W)
        return fail(KRETS_ERR_INVALID_ARGUMENT, "krets_batch_tran_noalloc: one CTA's FP64 fallback factors exceed "
                                                "the 16 MiB scratch");
      grid = std::min(grid, (int)(slots / W));
      fb = (double *)(base + lu_off);
    }
    const char *tenv = getenv("KRETS_REFINE_TOL");
    const double tol = tenv ? atof(tenv) : 1e-8;
    c->warps_per_cta = W;
    c->grid = grid;
    CU(cudaEventRecord(c->ev[2], c->stream));
    if (use_df)
      k_tran_warp_df<<<grid, 32 * W, smem, c->stream>>>(P, c->cfg, WL, d_values, n_inst, h, n_steps, method,
                                                       source_lag, d_x_out, d_inst_status, queue, hist, (float)tol);
    else
      kern<<<grid, 32 * W, smem, c->stream>>>(P, c->cfg, WL, d_values, n_inst, h, n_steps, method, source_lag, d_x_out,
                                             d_inst_status, queue, hist, fallbacks, fb, tol);
  }
  g_launches++;
  CU(cudaGetLastError());
  CU(cudaEventRecord(c->ev[3], c->stream));
  k_status_fold<<<std::max(1, std::min(1024, (n_inst + 255) / 256)), 256, 0, c->stream>>>(op_status, d_inst_status,
                                                                                         n_inst, any_op, any_tran);
  g_launches++;
  CU(cudaGetLastError());
  int any_h[2] = {0, 0};
  CU(cudaMemcpyAsync(any_h, any_op, sizeof any_h, cudaMemcpyDeviceToHost, c->stream));
  CU(cudaEventRecord(c->ev[1], c->stream));
  CU(cudaStreamSynchronize(c->stream));
  cudaEventElapsedTime(&c->kernel_ms, c->ev[2], c->ev[3]);
  cudaEventElapsedTime(&c->call_ms, c->ev[0], c->ev[1]);
  if (any_h[0]) return map_status(any_h[0], 0);
  return map_status(any_h[1], 1);
}

// ------------------------------------------------------------------ multi-circuit
krets_status krets_multi_create(int32_t n_circuits, const krets_element *elems, const int64_t *elem_offsets,
                                const int32_t *n_unknowns, int32_t method, double h, krets_multi **out) {
  if (!out || n_circuits <= 0 || !elems || !elem_offsets || !n_unknowns || !(h > 0) ||
      (method != KRETS_METHOD_BE && method != KRETS_METHOD_TR))
    return fail(KRETS_ERR_INVALID_ARGUMENT, "invalid arguments to krets_multi_create");
  *out = nullptr;
  int dev_count = 0;
  if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count == 0) {
    cudaGetLastError();
    return fail(KRETS_ERR_CUDA, "no CUDA device is available (this library has no CPU fallback)");
  }
  auto m = std::make_unique<krets_multi>();
  const int N = n_circuits;
  m->n_circ = N;
  m->method = method;
  m->h = h;
  m->n.assign(n_unknowns, n_unknowns + N);
  m->el_off.assign(elem_offsets, elem_offsets + N + 1);
  m->ne.resize(N);
  for (int c = 0; c < N; ++c) {
    const long long e0 = m->el_off[c], e1 = m->el_off[c + 1];
    if (e1 < e0 || m->n[c] <= 0) return fail(KRETS_ERR_INVALID_ARGUMENT, "circuit " + std::to_string(c) + ": bad sizes");
    m->ne[c] = (int)(e1 - e0);
    for (long long e = e0; e < e1; ++e) {
      const krets_element &x = elems[e];
      if (x.kind < KRETS_ELEM_R || x.kind > KRETS_ELEM_Q)
        return fail(KRETS_ERR_INVALID_ELEMENT, "circuit " + std::to_string(c) + ": unknown element kind");
      for (int v : {x.p, x.m, x.b, x.g})
        if (v < -1 || v >= m->n[c])
          return fail(KRETS_ERR_INVALID_ARGUMENT, "circuit " + std::to_string(c) + ": unknown index out of range");
    }
  }
  // f(j) for j = 0 .. count-1 on all host threads (a shared counter hands out the jobs)
  auto parallel_for = [](int count, const auto &f) {
    std::atomic<int> next{0};
    const int nt = std::max(1, std::min({(int)std::thread::hardware_concurrency(), 64, count}));
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t)
      th.emplace_back([&]() {
        for (int j; (j = next.fetch_add(1)) < count;) f(j);
      });
    for (auto &t : th) t.join();
  };
  // host symbolic pass of every circuit (DC and TRAN programs), on all host threads
  std::vector<Program> progs(2 * (size_t)N);
  std::vector<int> pst(2 * (size_t)N, 0);
  std::vector<std::string> pmsg(2 * (size_t)N);
  parallel_for(2 * N, [&](int j) {
    const int c = j / 2, mode = (j & 1) ? MODE_TRAN : MODE_DC;
    pst[j] = build_program(elems + m->el_off[c], m->ne[c], m->n[c], mode, method, h, 0.0, -1, progs[j], pmsg[j],
                           false, true);
  });
  for (int j = 0; j < 2 * N; ++j) {
    if (pst[j] != KRETS_OK) return fail(pst[j], "circuit " + std::to_string(j / 2) + ": " + pmsg[j]);
    bool nonlinear = false;
    for (long long e = m->el_off[j / 2]; e < m->el_off[j / 2 + 1]; ++e)
      nonlinear |= elems[e].kind == KRETS_ELEM_D || elems[e].kind == KRETS_ELEM_M || elems[e].kind == KRETS_ELEM_Q;
    if (nonlinear)
      return fail(KRETS_ERR_NOT_IMPLEMENTED, "circuit " + std::to_string(j / 2) +
                                                 ": the multi-circuit engine runs linear circuits (R, C, L, V, I)");
    if (!progs[j].sprog_ok) return fail(KRETS_ERR_INVALID_ARGUMENT, "circuit " + std::to_string(j / 2) + " too large");
  }
  // one device image for all programs
  CU(cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking));
  for (auto &e : m->ev) CU(cudaEventCreate(&e));
  const long long ne_total = m->el_off[N];
  CU(cudaMalloc(&m->d_el, sizeof(krets_element) * std::max(1ll, ne_total)));
  CU(cudaMemcpy(m->d_el, elems, sizeof(krets_element) * ne_total, cudaMemcpyHostToDevice));
  // The image of all programs (GBs for a large batch) is built on all host threads; its
  // staging copy is not zeroed first, since no kernel reads the padding between arrays.
  std::vector<ProgramImage> X(2 * (size_t)N);
  std::vector<size_t> off(2 * (size_t)N + 1, 0);
  parallel_for(2 * N, [&](int j) { image_extras(progs[j], X[j]); });
  for (int j = 0; j < 2 * N; ++j) off[j + 1] = off[j] + program_bytes(progs[j], X[j]);
  CU(cudaMalloc(&m->d_image, off[2 * N]));
  std::vector<DevProg> views(2 * (size_t)N);
  {
    std::unique_ptr<char[]> staging(new char[std::max<size_t>(off[2 * N], 1)]);
    parallel_for(2 * N, [&](int j) {
      const int c = j / 2;
      place_program(progs[j], X[j], elems + m->el_off[c], m->d_el + m->el_off[c], (char *)m->d_image + off[j],
                    staging.get() + off[j], views[j]);
    });
    CU(cudaMemcpy(m->d_image, staging.get(), off[2 * N], cudaMemcpyHostToDevice));
  }
  CU(cudaMalloc(&m->d_views, sizeof(DevProg) * views.size()));
  CU(cudaMemcpy(m->d_views, views.data(), sizeof(DevProg) * views.size(), cudaMemcpyHostToDevice));
  // size classes: the smallest shared-memory region that holds both phases of a circuit
  const long long smax = (long long)max_smem_optin();
  struct Spec { int G, W; };
  const Spec specs[] = {{32, 16}, {32, 8}, {64, 4}, {128, 2}, {128, 1}};
  for (const Spec &sp : specs) {
    MultiClass k;
    k.G = sp.G;
    k.W = sp.W;
    k.region = (smax / sp.W) & ~15ll;
    m->classes.push_back(k);
  }
  MultiClass kg;
  kg.G = 256;
  kg.W = 1;
  kg.global = true;
  m->classes.push_back(kg);
  std::vector<long long> need(N), need_g(N);
  m->nnz_lu_tr.resize(N);
  m->levels_tr.resize(N);
  for (int c = 0; c < N; ++c) {
    long long a = 0, g = 0;
    for (int ph = 0; ph < 2; ++ph) {
      const DevProg &V = views[2 * c + ph];
      a = std::max<long long>(a, multi_lay(V.nnz_lu, V.n, V.ndyn, V.ncap, V.ne, V.sp_off[5], V.n_bchunk).bytes);
      g = std::max<long long>(g, multi_lay(V.nnz_lu, V.n, V.ndyn, V.ncap, V.ne, 0, V.n_bchunk).bytes);
    }
    need[c] = a;
    need_g[c] = g;
    m->nnz_lu_tr[c] = views[2 * c + 1].nnz_lu;
    m->levels_tr[c] = views[2 * c + 1].nlev + views[2 * c + 1].nulev;
  }
  std::vector<int> order(N);
  for (int c = 0; c < N; ++c) order[c] = c;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return need[a] > need[b]; });
  for (int c : order) {
    // smallest fitting region: the classes are in increasing region size
    int pick = -1;
    for (size_t q = 0; q + 1 < m->classes.size(); ++q)
      if (m->classes[q].region >= need[c]) { pick = (int)q; break; }
    if (pick < 0) {
      pick = (int)m->classes.size() - 1;
      m->classes[pick].region = std::max(m->classes[pick].region, (long long)mlay_al16(need_g[c]));
    }
    m->classes[pick].items.push_back(c);
  }
  std::vector<int> all_items;
  long long gscratch_bytes = 0;
  for (auto &k : m->classes) {
    if (k.items.empty()) continue;
    CU(cudaStreamCreateWithFlags(&k.stream, cudaStreamNonBlocking));
    CU(cudaEventCreate(&k.done));
    int per_sm = 1;
    if (k.global) {
      // shared memory of a global-class group (half an SM's, two groups per SM): during the
      // steps a staging tile, x and the rhs coefficients, with the dense-block row slots at
      // the end; during the set-up the same bytes hold the factorisation's row staging
      // (8 warps x (dense row + sparse row)) or its tiles.  Without room for the step
      // layout, x stays in global memory.
      long long need = 0;
      for (int c : k.items)
        for (int ph = 0; ph < 2; ++ph) {
          const DevProg &V = views[2 * c + ph];
          const long long rows = mlay_al16(4ll * V.tail_m);
          const long long step = kStageBytes + mlay_al16(8ll * V.n) + mlay_al16(8ll * V.ndyn) + rows;
          long long stage = 0;
          if (V.tail_m) {
            const Program &H = progs[2 * c + ph];
            const long long cap = H.sprog[H.sp_off[12] + V.nlev - 1] >> 18;
            stage = 8 * (((2ll * V.tail_m + 3 * cap + 3) & ~3ll) * 4) + rows;
          }
          need = std::max(need, std::max(step, stage));
        }
      // three groups per SM (the kernel is built for 80 registers a thread) when their
      // shared memory fits a third of the SM's, else two: the class is latency bound, so
      // resident groups set its throughput (4096 uneven netlists: 3.5 s -> 3.0 s); four
      // would leave x in global memory and the dense-block tiles small, which is slower
      const long long third = (long long)(max_smem_per_sm() / 3) - 1024;
      per_sm = need <= third ? 3 : 2;
      k.x_smem = need <= (per_sm == 3 ? third : smax / 2);
      k.gsm = k.x_smem ? need : kStageBytes;
    }
    k.grid = std::max(1, std::min(((int)k.items.size() + k.W - 1) / k.W, per_sm * device_sm_count()));
    if (k.global) gscratch_bytes = k.region * k.grid * k.W;
    all_items.insert(all_items.end(), k.items.begin(), k.items.end());
  }
  CU(cudaMalloc(&m->d_items, sizeof(int) * all_items.size()));
  CU(cudaMemcpy(m->d_items, all_items.data(), sizeof(int) * all_items.size(), cudaMemcpyHostToDevice));
  CU(cudaMalloc(&m->d_queue, sizeof(int) * 16));
  CU(cudaMalloc(&m->d_status, sizeof(int) * N));
  CU(cudaMalloc(&m->d_xoff, sizeof(long long) * N));
  if (gscratch_bytes) CU(cudaMalloc(&m->gscratch, gscratch_bytes));
  *out = m.release();
  return KRETS_OK;
}

krets_status krets_multi_destroy(krets_multi *m) {
  delete m;
  return KRETS_OK;
}

krets_status krets_multi_info(const krets_multi *m, int64_t *info, int32_t cap) {
  if (!m || !info || cap < 4) return fail(KRETS_ERR_INVALID_ARGUMENT, "invalid arguments to krets_multi_info");
  long long sn = 0, snnz = 0, slev = 0;
  for (int c = 0; c < m->n_circ; ++c) {
    sn += m->n[c];
    snnz += m->nnz_lu_tr[c];
    slev += m->levels_tr[c];
  }
  std::vector<long long> v{m->n_circ, sn, snnz, slev};
  for (auto &k : m->classes) v.push_back((long long)k.items.size());
  for (auto &k : m->classes) v.push_back((long long)(1000.0 * k.ms));
  for (int i = 0; i < cap && i < (int)v.size(); ++i) info[i] = v[i];
  return KRETS_OK;
}

krets_status krets_multi_tran(krets_multi *m, int32_t n_steps, int32_t source_lag, double *x_out,
                              const int64_t *x_offsets, int32_t *circuit_status) {
  if (!m || n_steps < 0 || !x_out) return fail(KRETS_ERR_INVALID_ARGUMENT, "invalid arguments to krets_multi_tran");
  const int N = m->n_circ;
  std::vector<long long> xo(N);
  long long total = 0;
  for (int c = 0; c < N; ++c) {
    xo[c] = x_offsets ? x_offsets[c] : total;
    total = std::max(total, xo[c] + (long long)(n_steps + 1) * m->n[c]);
  }
  CU(cudaEventRecord(m->ev[0], m->stream));
  DevBuf tx;
  void *dx;
  krets_status s = dev_view(x_out, sizeof(double) * total, false, m->stream, tx, &dx);
  if (s) return s;
  CU(cudaMemcpyAsync(m->d_xoff, xo.data(), sizeof(long long) * N, cudaMemcpyHostToDevice, m->stream));
  CU(cudaMemsetAsync(m->d_queue, 0, sizeof(int) * 16, m->stream));
  CU(cudaMemsetAsync(m->d_status, 0, sizeof(int) * N, m->stream));
  CU(cudaEventRecord(m->ev[2], m->stream));
  // every size class on its own stream: CTAs of the next class fill SMs as a class drains
  int base = 0, qi = 0;
  for (auto &k : m->classes) {
    if (k.items.empty()) continue;
    CU(cudaStreamWaitEvent(k.stream, m->ev[2], 0));
    const int threads = k.G * k.W;
    const size_t smem = k.global ? (size_t)k.gsm * k.W : (size_t)(k.region * k.W);
    void (*kern)(const DevProg *, const int *, int, const long long *, long long, char *, int, int, double, int, int,
                 int, double *, int *, int *) = nullptr;
    if (k.global) kern = k_multi_tran<256, true>;
    else if (k.G == 32) kern = k_multi_tran<32, false>;
    else if (k.G == 64) kern = k_multi_tran<64, false>;
    else kern = k_multi_tran<128, false>;
    CU(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kern<<<k.grid, threads, smem, k.stream>>>(m->d_views, m->d_items + base, (int)k.items.size(), m->d_xoff, k.region,
                                             m->gscratch, (int)k.gsm, k.x_smem ? 1 : 0, m->h, n_steps, m->method,
                                             source_lag, (double *)dx, m->d_status, m->d_queue + qi);
    g_launches++;
    CU(cudaGetLastError());
    CU(cudaEventRecord(k.done, k.stream));
    CU(cudaStreamWaitEvent(m->stream, k.done, 0));
    base += (int)k.items.size();
    ++qi;
  }
  CU(cudaEventRecord(m->ev[3], m->stream));
  if (tx.p) CU(cudaMemcpyAsync(x_out, dx, sizeof(double) * total, cudaMemcpyDeviceToHost, m->stream));
  std::vector<int> st(N);
  CU(cudaMemcpyAsync(st.data(), m->d_status, sizeof(int) * N, cudaMemcpyDeviceToHost, m->stream));
  CU(cudaEventRecord(m->ev[1], m->stream));
  CU(cudaStreamSynchronize(m->stream));
  cudaEventElapsedTime(&m->kernel_ms, m->ev[2], m->ev[3]);
  cudaEventElapsedTime(&m->call_ms, m->ev[0], m->ev[1]);
  for (auto &k : m->classes)
    if (!k.items.empty()) cudaEventElapsedTime(&k.ms, m->ev[2], k.done);
  int any = 0;
  for (int c = 0; c < N; ++c) {
    if (circuit_status) circuit_status[c] = map_status(st[c], 0);
    any |= st[c];
  }
  return map_status(any, 0);
}

int32_t krets_direct_host_access(void) { return direct_host_access() ? 1 : 0; }

krets_status krets_multi_last_timing(const krets_multi *m, float *kernel_ms, float *call_ms) {
  if (!m) return fail(KRETS_ERR_INVALID_ARGUMENT, "null multi-circuit handle");
  if (kernel_ms) *kernel_ms = m->kernel_ms;
  if (call_ms) *call_ms = m->call_ms;
  return KRETS_OK;
}

}  // extern "C"
