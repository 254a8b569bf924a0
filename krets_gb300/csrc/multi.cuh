// Multi-circuit transient: one launch runs the operating point and the transient of many
// distinct netlists (different topologies and sizes).  Each circuit has two programs from
// the host symbolic pass (DC for the operating point, TRAN for the steps), all in one
// device image with an array of program views; the programs carry no factorisation update
// list (its size grows with the factorisation work), the LU is formed by merging rows.
// A group of G threads takes a circuit from a device work queue and runs both phases with
// the double-float direct engine:
//   phase 0: stamp and factor the DC matrix, solve the operating point, write row 0;
//   phase 1: stamp and factor the transient matrix, step from row 0.
// The circuit's step program and working arrays sit in the group's region of shared
// memory (SMEM variants, one launch per region size) or, for circuits too large for it,
// in a per-group region of global memory with the step program read in place (GLOBAL).
#pragma once

#include "warp_kernels.cuh"

namespace krets {

// Working arrays of one circuit phase inside its region: a 16-byte header (queue slot
// and status words), the staged step program (SMEM only), then the instance arrays.
struct MLay {
  int sp, lu, x, cdyn, cb, icap, bpart, coef64, bytes;
};

__host__ __device__ inline int mlay_al16(long long v) { return (int)((v + 15) & ~15ll); }

__host__ __device__ inline MLay multi_lay(int nnz_lu, int n, int ndyn, int ncap, int ne, int sp_words, int n_bchunk) {
  MLay L;
  long long cur = 16;
  L.sp = (int)cur;
  cur = mlay_al16(cur + 4ll * sp_words);
  L.lu = (int)cur;
  cur = mlay_al16(cur + 8ll * nnz_lu);
  L.x = (int)cur;
  cur = mlay_al16(cur + 8ll * n);
  L.cdyn = (int)cur;
  cur = mlay_al16(cur + 8ll * ndyn);
  L.cb = (int)cur;
  cur = mlay_al16(cur + 8ll * ndyn);
  L.icap = (int)cur;
  cur = mlay_al16(cur + 8ll * ncap);
  L.bpart = (int)cur;  // partial sums of the dense block's border chunks
  cur = mlay_al16(cur + 8ll * n_bchunk);
  L.coef64 = L.x;  // set-up scratch over x .. bpart (+ padding if needed)
  if (cur - L.x < 8ll * ne) cur = L.x + mlay_al16(8ll * ne);
  L.bytes = (int)cur;
  return L;
}

// GLOBAL: shared memory per group = a 32 x 33 staging tile for the diagonal blocks of the
// dense trailing block, then (x_smem) the solution and rhs-coefficient vectors, whose
// gathers are the latency-critical accesses; the LU and the step program stay in global
// memory.
constexpr int kStageBytes = 32 * 33 * 8;

// GLOBAL: one 256-thread group per CTA, three CTAs per SM (80 registers a thread).
template <int G, bool GLOBAL>
__global__ void __launch_bounds__(GLOBAL ? 256 : 512, GLOBAL ? 3 : 1)
    k_multi_tran(const DevProg *__restrict__ progs, const int *__restrict__ items, int n_items,
                 const long long *__restrict__ x_off, long long region_bytes, char *gscratch, int gsm_bytes,
                 int x_smem, double h, int n_steps, int method, int lag, double *x_out, int *circ_status,
                 int *queue) {
  extern __shared__ __align__(16) char smem[];
  const int gl = threadIdx.x % G, gid = threadIdx.x / G;
  const int W = blockDim.x / G;
  char *region = GLOBAL ? gscratch + ((long long)blockIdx.x * W + gid) * region_bytes
                        : smem + (long long)gid * region_bytes;
  char *gsm = smem + (long long)gid * gsm_bytes;  // GLOBAL only
  int *slot = reinterpret_cast<int *>(region);
  while (true) {
    if (gl == 0) slot[0] = atomicAdd(queue, 1);
    gsync<G>(gid);
    const int item = slot[0];
    gsync<G>(gid);
    if (item >= n_items) break;
    const int c = items[item];
    double *out = x_out + x_off[c];
    int st = 0;
    for (int phase = 0; phase < 2; ++phase) {
      const DevProg P = progs[2 * c + phase];
      const int spw = GLOBAL ? 0 : P.sp_off[5];
      const MLay L = multi_lay(P.nnz_lu, P.n, P.ndyn, P.ncap, P.ne, spw, P.n_bchunk);
      if (!GLOBAL) {
        const int4 *src = reinterpret_cast<const int4 *>(P.sprog);
        int4 *dst = reinterpret_cast<int4 *>(region + L.sp);
        for (int i = gl; i < spw / 4; i += G) dst[i] = src[i];
        gsync<G>(gid);
      }
      SProg S = sprog_view(P, GLOBAL ? P.sprog : reinterpret_cast<const int *>(region + L.sp));
      S.bpart = reinterpret_cast<df *>(region + L.bpart);
      const bool xs = GLOBAL && x_smem;
      if (GLOBAL) {
        S.dense_stage = reinterpret_cast<df *>(gsm);
        if (xs && P.tail_m) {
          // slots of the dense-block rows, at the end of the group's shared memory
          int *rows = reinterpret_cast<int *>(gsm + gsm_bytes - mlay_al16(4ll * P.tail_m));
          for (int i = gl; i < P.tail_m; i += G) rows[i] = P.lu_rowptr[P.tail0 + i + 1] - P.tail_m;
          gsync<G>(gid);
          S.dense_rows = rows;
        }
      }
      df *lu = reinterpret_cast<df *>(region + L.lu);
      double *lu64 = reinterpret_cast<double *>(region + L.lu);
      df *x = reinterpret_cast<df *>(xs ? gsm + kStageBytes : region + L.x);
      df *cdyn = reinterpret_cast<df *>(region + L.cdyn);
      df *cb = reinterpret_cast<df *>(xs ? gsm + kStageBytes + mlay_al16(8ll * P.n) : region + L.cb);
      df *icap = reinterpret_cast<df *>(region + L.icap);
      double *coef64 = reinterpret_cast<double *>(region + L.coef64);
      // global class: the factorisation's column map (sparse part) and 32 x tw tiles (dense
      // block) use the shared memory that x and the rhs coefficients take later (free
      // during the set-up)
      const long long tile_bytes = xs ? gsm_bytes - mlay_al16(4ll * P.tail_m) : kStageBytes;
      const int tw = (int)min(128ll, (tile_bytes / (32 * 8)) / 32 * 32);
      st |= dfd_setup<G, GLOBAL ? 2 : 1>(P, S, nullptr, h, method, lu, lu64, coef64, cdyn, gl, gid,
                                         reinterpret_cast<double *>(gsm), tw, tile_bytes);
      if (gany<G>((st & (KS_SINGULAR | KS_NONFINITE | KS_NOTIMPL)) != 0, gid)) break;
      if (phase == 0) {
        // operating point: sources at their DC values (op.rs: capacitors removed,
        // inductors as shorts through their branch rows)
        for (int d = gl; d < P.ndyn; d += G) {
          const int4 dd = S.dyn[d];
          const int kind = (int)((unsigned)dd.x >> 24);
          cb[d] = (kind == KRETS_ELEM_V || kind == KRETS_ELEM_I) ? df_from_double(P.el[dd.x & 0xffffff].value)
                                                                 : df{0.f, 0.f};
        }
        gsync<G>(gid);
        for (int k = gl; k < P.n; k += G) {
          df acc{0.f, 0.f};
          for (int u = S.bd_ptr[k]; u < S.bd_ptr[k + 1]; ++u) {
            const int code = S.bd_op[u];
            acc = df_add(acc, (code & 1) ? df_neg(cb[code >> 1]) : cb[code >> 1]);
          }
          x[k] = acc;
        }
        gsync<G>(gid);
        df_solve<G, false, GLOBAL ? 0 : G>(S, lu, x, gl, gid, -1);
        df_solve<G, true, GLOBAL ? 0 : G>(S, lu, x, gl, gid, -1);
        for (int k = gl; k < P.n; k += G) {
          const double v = df_to_double(x[S.qinv[k]]);
          if (!isfinite(v)) st |= KS_NONFINITE;
          out[k] = v;
        }
        gsync<G>(gid);  // row 0 complete before the transient phase reads it
      } else {
        for (int k = gl; k < P.n; k += G) x[k] = df_from_double(out[P.q[k]]);
        for (int d = gl; d < P.ncap; d += G) icap[d] = df{0.f, 0.f};
        gsync<G>(gid);
        st |= dfd_steps<G, GLOBAL ? 0 : G>(P, S, lu, x, cdyn, cb, icap, nullptr, h, n_steps, method, lag, out, -1, -1,
                                          false, gl, gid);
      }
    }
    if (gl == 0) slot[1] = 0;
    gsync<G>(gid);
    if (st) atomicOr(&slot[1], st);
    gsync<G>(gid);
    if (gl == 0 && circ_status) circ_status[c] = slot[1];
  }
}

}  // namespace krets
