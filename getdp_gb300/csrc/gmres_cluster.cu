// Batched GMRES / FGMRES with one thread-block cluster per system and the
// whole solve of every system in one launch.
//
// The systems of a batch (the diagonal blocks of one matrix, as in
// gmres_batch.cu) are independent, so nothing has to cross from one system
// to another while they iterate: a cluster of 1 to 16 CTAs (on as many SMs)
// takes a system from a queue (largest first), runs its restart cycles and
// Arnoldi steps to the end, and takes the next.  Within a cluster the rows
// are split between the CTAs; the steps that need rows of other CTAs (the
// ILU(0) sweeps level by level, the product with the preconditioned vector,
// the restart residual) follow a cluster barrier, and every sum (the
// Gram-Schmidt dot products, norms) is formed per CTA in a fixed order, left
// in the CTA's shared memory, and read by every CTA of the cluster through
// distributed shared memory in rank order, so that every CTA holds the same
// sums and runs the same scalar recurrences (Hessenberg column, Givens
// rotations, stopping tests) on its own copy: no launch per step, no
// grid-wide synchronisation, no host round trip.
//
// The iteration is the one of gmres_batch.cu and gmres.cu: right
// preconditioning, restart residual, classical Gram-Schmidt with the
// selective second pass (a second pass when the first removed more than
// 98 % of ||w||^2, mgsro's constant, iters.f:3475), Givens rotations
// (iters.f:3235-3273), Sparskit's stopping test on the rotated residual and
// its codes (iters.f:1912-2219 GMRES, :2522-2806 FGMRES).  The ILU(0)
// factor and its level schedule are the ones of gmres.cu, cut into the
// systems (ilu_sys_levels); a sweep's rows and arithmetic are those of
// lusol (ilut.F:2297-2347), in FP64 or with the FP32 factor.
//
// Cross-CTA data in global memory (vectors written by other CTAs of the
// cluster) is read through L2 (ld.global.cg) after a cluster barrier
// (barrier.cluster arrive.release / wait.acquire).  Every branch around a
// barrier depends only on values that all CTAs of the cluster hold alike,
// and every loop is bounded (restart cycles by the iteration cap, steps by
// the Krylov size, systems by the queue).
#include <cooperative_groups.h>

#include <algorithm>
#include <vector>

#include "krylov.cuh"

namespace cg = cooperative_groups;

namespace gb {

// CTAs per cluster (one cluster per system): Batch_Kernel 1, 2, 4, 8 (the
// portable maximum) or 16 (a non-portable size this GPU allows).  Measured
// on 512 complex systems of 1,922..51,842 rows (ILU(0)-GMRES(40) in the
// multicolour order, FP64 / FP32 factor): 1 CTA 2.32 / 2.07 s, 2 1.29 /
// 1.14, 4 0.958 / 0.856, 8 1.11 / 0.99, against 1.19 / 1.235 s for the
// per-kernel form: few CTAs leave the largest systems' steps to one or two
// SMs, many CTAs leave fewer systems running at once and make each cluster
// barrier dearer.  256-thread CTAs measured the same at the same threads
// per system (8 CTAs: 0.938 / 0.843 s) and slower at fewer (4 CTAs: 1.22 /
// 1.10 s)
constexpr int kCThreads = 512;
constexpr int kCWarps = kCThreads / 32;
constexpr int kCMaxKrylov = 64;
// most levels of one system in either triangular sweep (one cluster
// barrier each); systems in GetDP's own order (~2n levels on an n x n grid)
// take the chunked batched solver
constexpr int kCMaxLevels = 64;

struct CState {
  double tol, res, res0, res6, scale, nrm0, rr;
  int its, status, active, cycle, first, k, did_cycle, breakdown, reorth;
};

struct CArgs {
  int nsys, m, maxit, flexible, precond;
  double rtol;
  const int *order, *off;
  int *queue;
  const int *rowptr, *col;
  const double *val, *rhs;
  double *x;
  const int *diag;
  const void *lu, *inv;
  const int *lrows, *urows, *llev, *ulev, *llb, *ulb;
  // multicolour order: system p's vertices of colour c are
  // [voff[p (ncol + 1) + c], voff[p (ncol + 1) + c + 1]), bs rows each
  // (ncol = 0: the level lists above)
  int ncol, bs;
  const int *voff;
  double *Vb, *Z, *zt, *u;
  float *t32;
  size_t ldv;
  int *out_status, *out_its;
  double *out_res, *out_rr, *out_bb;
};

// the sums over the cluster's CTAs, in rank order, of the nv partials each
// CTA left in buf: every CTA gets the same values in out
template <int CS>
__device__ __forceinline__ void cluster_sum(cg::cluster_group &cl, double *buf, int nv,
                                            double *out)
{
  cl.sync();
  for(int j = threadIdx.x; j < nv; j += kCThreads) {
    double s = 0.;
#pragma unroll
    for(int r = 0; r < CS; r++) s += cl.map_shared_rank(buf, r)[j];
    out[j] = s;
  }
  __syncthreads();
}

// s - sum_k a[k] x[col[k]] over k = k0, k0 + step, ... < k1, in that order
// (lusol's and amux's accumulation order), with the column indices and
// values of up to eight entries loaded before their gathers, so that a
// thread has eight loads in flight instead of a chain of dependent ones
template <int STEP, bool SUB, typename T, typename X>
__device__ __forceinline__ T row_acc(int k0, int k1, const int *__restrict__ col,
                                     const T *__restrict__ a, const X *x, T s)
{
  for(int kb = k0; kb < k1; kb += 4 * STEP) {
    int c[4];
    T v[4];
    X xv[4];
#pragma unroll
    for(int u = 0; u < 4; u++) {
      int k = kb + u * STEP;
      c[u] = k < k1 ? col[k] : 0;
      v[u] = k < k1 ? a[k] : (T)0;
    }
#pragma unroll
    for(int u = 0; u < 4; u++)
      if(kb + u * STEP < k1) xv[u] = __ldcg(x + c[u]);
#pragma unroll
    for(int u = 0; u < 4; u++)
      if(kb + u * STEP < k1) {
        if(SUB)
          s = s - v[u] * xv[u];
        else
          s += v[u] * xv[u];
      }
  }
  return s;
}

// the sum over the cluster's CTAs and their warps, in (rank, warp) order, of
// the one partial per warp each CTA left in buf[0 .. kCWarps): every CTA
// gets the same value in out[0] (no CTA-wide sum first)
template <int CS>
__device__ __forceinline__ void cluster_sum_warps(cg::cluster_group &cl, double *buf,
                                                  double *out)
{
  cl.sync();
  if(threadIdx.x < 32) {
    double s = 0.;
    for(int r = 0; r < CS; r++) {
      double v = threadIdx.x < kCWarps ? cl.map_shared_rank(buf, r)[threadIdx.x] : 0.;
      s += warp_sum(v);  // lane 0 holds the rank's sum
    }
    if(threadIdx.x == 0) out[0] = s;
  }
  __syncthreads();
}

// w = A z on the rows [lo, hi) (two lanes per row, as k_b_spmv); with RES,
// w = rhs - A z and the partial ||w||^2 (and ||rhs||^2 in bb)
template <int RES>
__device__ __forceinline__ double c_spmv(const CArgs &P, int lo, int hi, const double *z,
                                         double *w, double *bb)
{
  const int l2 = threadIdx.x & 1, sub = threadIdx.x >> 1;
  double acc = 0., accb = 0.;
  for(int i = lo + sub; i - sub < hi; i += kCThreads / 2) {
    double s = 0.;
    if(i < hi) s = row_acc<2, false>(P.rowptr[i] + l2, P.rowptr[i + 1], P.col, P.val, z, s);
    s += __shfl_down_sync(0xffffffffu, s, 1, 2);
    if(l2 == 0 && i < hi) {
      if(RES) {
        double ri = P.rhs[i] - s;
        if(w) w[i] = ri;
        acc += ri * ri;
        accb += P.rhs[i] * P.rhs[i];
      }
      else
        w[i] = s;
    }
  }
  if(bb) *bb = accb;
  return acc;
}

// partial <V_j, w> over the rows [lo, hi) for j < kk, one warp per column
// (a fixed order per column), into buf[j]
__device__ __forceinline__ void c_dots(const CArgs &P, int lo, int hi, const double *w,
                                       int kk, double *buf)
{
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for(int j = warp; j < kk; j += kCWarps) {
    const double *vj = P.Vb + (size_t)j * P.ldv;
    double s = 0.;
#pragma unroll 4
    for(int i = lo + lane; i < hi; i += 32) s += __ldcg(vj + i) * __ldcg(w + i);
    s = warp_sum(s);
    if(lane == 0) buf[j] = s;
  }
}

// w -= sum_{j<k} h_j V_j on the rows [lo, hi); the partial ||w||^2
__device__ __forceinline__ double c_update(const CArgs &P, int lo, int hi, double *w,
                                           const double *h, int k)
{
  double v = 0.;
  for(int i = lo + threadIdx.x; i < hi; i += kCThreads) {
    // four independent FMA chains (as k_b_update)
    double s0 = 0., s1 = 0., s2 = 0., s3 = 0.;
    int j = 0;
    for(; j + 3 < k; j += 4) {
      s0 += h[j] * __ldcg(P.Vb + (size_t)j * P.ldv + i);
      s1 += h[j + 1] * __ldcg(P.Vb + (size_t)(j + 1) * P.ldv + i);
      s2 += h[j + 2] * __ldcg(P.Vb + (size_t)(j + 2) * P.ldv + i);
      s3 += h[j + 3] * __ldcg(P.Vb + (size_t)(j + 3) * P.ldv + i);
    }
    for(; j < k; j++) s0 += h[j] * __ldcg(P.Vb + (size_t)j * P.ldv + i);
    double wi = __ldcg(w + i) - ((s0 + s1) + (s2 + s3));
    w[i] = wi;
    v += wi * wi;
  }
  return v;
}

// dst = M^-1 src for system p: the ILU(0) sweeps level by level, each
// level's rows split over the cluster (a barrier after each level), or a
// copy without a preconditioner.  src must be complete (all CTAs) on entry;
// dst is complete on return.
template <typename T, int CS>
__device__ void c_precond(const CArgs &P, cg::cluster_group &cl, int p, int rank, int lo,
                          int hi, const double *src, double *dst)
{
  if(!P.precond) {
    for(int i = lo + threadIdx.x; i < hi; i += kCThreads) dst[i] = __ldcg(src + i);
    cl.sync();
    return;
  }
  const T *lu = (const T *)P.lu, *inv = (const T *)P.inv;
  cl.sync();  // src written by every CTA
  if(P.ncol > 0) {
    // colour by colour: a colour's vertices share no entry, so they are
    // independent; a vertex's bs rows (a complex unknown's two real rows)
    // go in order in one thread, forward first to last, backward last to
    // first: one barrier per colour instead of one per level
    const int *vo = P.voff + (size_t)p * (P.ncol + 1);
    const int bs = P.bs;
    for(int c = 0; c < P.ncol; c++) {
      const int a = vo[c], cnt = vo[c + 1] - a;
      if(cnt == 0) continue;  // the same for every CTA
      const int t0 = a + (int)((long long)cnt * rank / CS);
      const int t1 = a + (int)((long long)cnt * (rank + 1) / CS);
      for(int v = t0 + threadIdx.x; v < t1; v += kCThreads)
        for(int q = 0; q < bs; q++) {
          const int i = v * bs + q;
          if constexpr(sizeof(T) == 8)
            dst[i] = row_acc<1, true>(P.rowptr[i], P.diag[i], P.col, lu,
                                      (const double *)dst, __ldcg(src + i));
          else
            P.t32[i] = row_acc<1, true>(P.rowptr[i], P.diag[i], P.col, lu,
                                        (const float *)P.t32, (float)__ldcg(src + i));
        }
      cl.sync();
    }
    for(int c = P.ncol - 1; c >= 0; c--) {
      const int a = vo[c], cnt = vo[c + 1] - a;
      if(cnt == 0) continue;
      const int t0 = a + (int)((long long)cnt * rank / CS);
      const int t1 = a + (int)((long long)cnt * (rank + 1) / CS);
      for(int v = t0 + threadIdx.x; v < t1; v += kCThreads)
        for(int q = bs - 1; q >= 0; q--) {
          const int i = v * bs + q;
          const int ke = P.rowptr[i + 1];
          if constexpr(sizeof(T) == 8) {
            double s = row_acc<1, true>(P.diag[i] + 1, ke, P.col, lu, (const double *)dst,
                                        __ldcg(dst + i));
            dst[i] = inv[i] * s;
          }
          else {
            float s = row_acc<1, true>(P.diag[i] + 1, ke, P.col, lu, (const float *)P.t32,
                                       __ldcg(P.t32 + i));
            float w = inv[i] * s;
            P.t32[i] = w;
            dst[i] = (double)w;
          }
        }
      cl.sync();
    }
    return;
  }
  for(int l = P.llb[p]; l + 1 < P.llb[p + 1]; l++) {
    const int a = P.llev[l], cnt = P.llev[l + 1] - a;
    const int t0 = a + (int)((long long)cnt * rank / CS);
    const int t1 = a + (int)((long long)cnt * (rank + 1) / CS);
    for(int t = t0 + threadIdx.x; t < t1; t += kCThreads) {
      const int i = P.lrows[t];
      const int ke = P.diag[i];
      if constexpr(sizeof(T) == 8)
        dst[i] = row_acc<1, true>(P.rowptr[i], ke, P.col, lu, (const double *)dst,
                                  __ldcg(src + i));
      else
        P.t32[i] = row_acc<1, true>(P.rowptr[i], ke, P.col, lu, (const float *)P.t32,
                                    (float)__ldcg(src + i));
    }
    cl.sync();
  }
  for(int l = P.ulb[p]; l + 1 < P.ulb[p + 1]; l++) {
    const int a = P.ulev[l], cnt = P.ulev[l + 1] - a;
    const int t0 = a + (int)((long long)cnt * rank / CS);
    const int t1 = a + (int)((long long)cnt * (rank + 1) / CS);
    for(int t = t0 + threadIdx.x; t < t1; t += kCThreads) {
      const int i = P.urows[t];
      const int ke = P.rowptr[i + 1];
      if constexpr(sizeof(T) == 8) {
        double s = row_acc<1, true>(P.diag[i] + 1, ke, P.col, lu, (const double *)dst,
                                    __ldcg(dst + i));
        dst[i] = inv[i] * s;
      }
      else {
        float s = row_acc<1, true>(P.diag[i] + 1, ke, P.col, lu, (const float *)P.t32,
                                   __ldcg(P.t32 + i));
        float v = inv[i] * s;
        P.t32[i] = v;
        dst[i] = (double)v;
      }
    }
    cl.sync();
  }
}

template <typename T, int CS>
__global__ void __launch_bounds__(kCThreads, 1024 / kCThreads) k_c_solve(CArgs P)
{
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (int)cl.block_rank();
  const int tid = threadIdx.x;
  const int m = P.m;
  __shared__ double sH[(kCMaxKrylov + 1) * kCMaxKrylov];  // column-major, ld m + 1
  __shared__ double scs[kCMaxKrylov], ssn[kCMaxKrylov], sy[kCMaxKrylov];
  __shared__ double sg[kCMaxKrylov + 1], sh1[kCMaxKrylov + 1], sdot[kCMaxKrylov + 1];
  __shared__ double xbuf[2][kCMaxKrylov + 2];  // partials read by the other CTAs
  __shared__ CState S;
  __shared__ int s_q;
  int xb = 0;

  for(int guard = 0; guard <= P.nsys; guard++) {
    if(rank == 0 && tid == 0) s_q = atomicAdd(P.queue, 1);
    cl.sync();
    const int q = *cl.map_shared_rank(&s_q, 0);
    cl.sync();  // every CTA has read the ticket before rank 0 takes the next
    if(q >= P.nsys) break;
    const int p = P.order[q];
    const int r0 = P.off[p], np = P.off[p + 1] - r0;
    const int lo = r0 + (int)((long long)np * rank / CS);
    const int hi = r0 + (int)((long long)np * (rank + 1) / CS);
    if(tid == 0) {
      memset(&S, 0, sizeof(S));
      S.active = 1;
      S.first = 1;
      S.status = 1;
    }
    __syncthreads();

    for(int cyc = 0; S.active && cyc <= P.maxit + 1; cyc++) {
      // restart: r = b - A x into V_0, ||r||
      cl.sync();  // x complete
      {
        double rr = warp_sum(c_spmv<1>(P, lo, hi, P.x, P.Vb, nullptr));
        if((tid & 31) == 0) xbuf[xb][tid >> 5] = rr;
        cluster_sum_warps<CS>(cl, xbuf[xb], sdot);
        xb ^= 1;
      }
      if(tid == 0) {
        S.its += 1;
        double alpha = sqrt(sdot[0]);
        if(S.first) {
          S.tol = P.rtol * alpha + 0.0;
          S.res0 = alpha;
          S.first = 0;
        }
        S.res = alpha;
        sg[0] = alpha;
        S.k = 0;
        S.did_cycle = 0;
        S.breakdown = 0;
        if(alpha <= S.tol) {
          S.status = 0;
          S.res6 = alpha;
          S.active = 0;
          S.cycle = 0;
        }
        else {
          S.scale = 1. / alpha;
          S.cycle = 1;
        }
      }
      __syncthreads();
      if(!S.cycle) break;  // converged at the restart
      for(int i = lo + tid; i < hi; i += kCThreads) P.Vb[i] = S.scale * P.Vb[i];

      for(int k = 1; k <= m && S.cycle; k++) {
        double *vk = P.Vb + (size_t)(k - 1) * P.ldv;
        double *w = P.Vb + (size_t)k * P.ldv;
        double *z = P.flexible ? P.Z + (size_t)(k - 1) * P.ldv : P.zt;
        c_precond<T, CS>(P, cl, p, rank, lo, hi, vk, z);
        c_spmv<0>(P, lo, hi, z, w, nullptr);
        __syncthreads();
        // first Gram-Schmidt pass: <V_j, w> for j < k and <w, w>
        c_dots(P, lo, hi, w, k + 1, xbuf[xb]);
        cluster_sum<CS>(cl, xbuf[xb], k + 1, sdot);
        xb ^= 1;
        if(tid == 0) {
          S.nrm0 = sdot[k];
          if(!(S.nrm0 > 0. && 1. / S.nrm0 > 0.)) {
            // mgsro's zero (-1) or abnormal (-2) norm: the cycle ends as a
            // break-down, the step's column unused
            S.breakdown = (S.nrm0 <= 0.) ? -1 : -2;
            S.its += 1;
            S.cycle = 0;
            S.reorth = 0;
          }
        }
        if(tid < k) {
          sh1[tid] = sdot[tid];
          sH[(k - 1) * (m + 1) + tid] = sdot[tid];
        }
        __syncthreads();
        if(!S.cycle) break;
        {
          double v = warp_sum(c_update(P, lo, hi, w, sh1, k));
          if((tid & 31) == 0) xbuf[xb][tid >> 5] = v;
          cluster_sum_warps<CS>(cl, xbuf[xb], sdot);
          xb ^= 1;
        }
        if(tid == 0) {
          S.rr = sdot[0];
          S.reorth = !(S.rr >= 0.02 * S.nrm0);
        }
        __syncthreads();
        if(S.reorth) {
          // second pass
          c_dots(P, lo, hi, w, k, xbuf[xb]);
          cluster_sum<CS>(cl, xbuf[xb], k, sdot);
          xb ^= 1;
          if(tid < k) sH[(k - 1) * (m + 1) + tid] = sh1[tid] + sdot[tid];
          __syncthreads();
          double v = warp_sum(c_update(P, lo, hi, w, sdot, k));
          if((tid & 31) == 0) xbuf[xb][tid >> 5] = v;
          cluster_sum_warps<CS>(cl, xbuf[xb], sdot);
          xb ^= 1;
          if(tid == 0) S.rr = sdot[0];
          __syncthreads();
        }
        // end of the Arnoldi step: h(k+1,k), rotations, stopping test
        if(tid == 0) {
          S.its += 1;
          double *Hc = sH + (size_t)(k - 1) * (m + 1);
          double nrm = sqrt(S.rr);
          Hc[k] = nrm;
          S.k = k;
          S.did_cycle = 1;
          if(!(nrm > 0.)) {
            S.breakdown = -3;
            S.cycle = 0;
          }
          else {
            for(int i = 0; i < k - 1; i++) {
              double a = Hc[i], c = scs[i], s = ssn[i];
              Hc[i] = c * a + s * Hc[i + 1];
              Hc[i + 1] = c * Hc[i + 1] - s * a;
            }
            double c, s;
            givens_dev(&Hc[k - 1], &Hc[k], &c, &s);
            scs[k - 1] = c;
            ssn[k - 1] = s;
            double alpha = -s * sg[k - 1];
            sg[k - 1] = c * sg[k - 1];
            sg[k] = alpha;
            alpha = fabs(alpha);
            S.res = alpha;
            S.scale = 1. / nrm;
            if(!(k < m && !(alpha <= S.tol) && (P.maxit <= 0 || S.its < P.maxit)))
              S.cycle = 0;
          }
        }
        __syncthreads();
        if(S.cycle)
          for(int i = lo + tid; i < hi; i += kCThreads) w[i] = S.scale * w[i];
      }

      // end of the cycle: H y = g (upper triangular), then the update.
      // Thread 0 changes S below: every thread takes what it branches on
      // first, and a barrier separates the two (a thread that read S after
      // the change would leave the cluster barriers of the others)
      const int dc = S.did_cycle;
      __syncthreads();
      if(dc) {
        if(tid == 0) {
          int k = S.k;
          while(k > 0 && sH[(k - 1) * (m + 1) + k - 1] == 0.) k--;
          if(k == 0) {
            S.status = -3;
            S.breakdown = -4;
            S.active = 0;
            S.did_cycle = 0;
          }
          else {
            S.k = k;
            for(int i = k - 1; i >= 0; i--) {
              double t = sg[i];
              for(int j = i + 1; j < k; j++) t -= sH[j * (m + 1) + i] * sy[j];
              sy[i] = t / sH[i * (m + 1) + i];
            }
          }
        }
        __syncthreads();
      }
      const int upd = S.active && S.did_cycle;
      __syncthreads();
      if(upd) {
        const int k = S.k;
        if(P.flexible) {
          for(int i = lo + tid; i < hi; i += kCThreads) {
            double s = P.x[i];
            for(int j = 0; j < k; j++) s += sy[j] * __ldcg(P.Z + (size_t)j * P.ldv + i);
            P.x[i] = s;
          }
        }
        else {
          for(int i = lo + tid; i < hi; i += kCThreads) {
            double s = 0.;
            for(int j = 0; j < k; j++) s += sy[j] * __ldcg(P.Vb + (size_t)j * P.ldv + i);
            P.u[i] = s;
          }
          c_precond<T, CS>(P, cl, p, rank, lo, hi, P.u, P.zt);
          for(int i = lo + tid; i < hi; i += kCThreads) P.x[i] += __ldcg(P.zt + i);
        }
      }
      __syncthreads();
      // the restart decision
      if(tid == 0 && S.active) {
        S.res6 = S.res;
        if(S.breakdown != 0) {
          S.status = -3;
          S.active = 0;
        }
        else {
          bool more = (S.its < P.maxit || P.maxit <= 0) && (S.res6 > S.tol);
          if(!more) {
            if(S.res6 <= S.tol)
              S.status = 0;
            else if(S.its >= P.maxit && P.maxit > 0)
              S.status = -1;
            else
              S.status = -10;
            S.active = 0;
          }
        }
      }
      __syncthreads();
    }

    // the system's true residual ||b - A x|| and ||b||
    cl.sync();
    {
      double bb = 0.;
      double rr = c_spmv<1>(P, lo, hi, P.x, nullptr, &bb);
      rr = block_sum<double, kCThreads>(rr);
      bb = block_sum<double, kCThreads>(bb);
      if(tid == 0) {
        xbuf[xb][0] = rr;
        xbuf[xb][1] = bb;
      }
      cluster_sum<CS>(cl, xbuf[xb], 2, sdot);
      xb ^= 1;
    }
    if(rank == 0 && tid == 0) {
      P.out_status[p] = S.active ? -1 : S.status;
      P.out_its[p] = S.its;
      P.out_res[p] = S.res6;
      P.out_rr[p] = sdot[0];
      P.out_bb[p] = sdot[1];
    }
    __syncthreads();
  }
}

template <typename T, int CS>
static int launch_c(const CArgs &a, cudaStream_t st, int *nclusters)
{
  if(CS > 8 &&
     cudaFuncSetAttribute(k_c_solve<T, CS>, cudaFuncAttributeNonPortableClusterSizeAllowed,
                          1) != cudaSuccess) {
    cudaGetLastError();
    *nclusters = 0;
    return GB300_OK;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = CS;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.blockDim = dim3(kCThreads, 1, 1);
  cfg.dynamicSmemBytes = 0;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cfg.gridDim = dim3(CS, 1, 1);
  int nc = 0;
  cudaError_t e = cudaOccupancyMaxActiveClusters(&nc, (void *)k_c_solve<T, CS>, &cfg);
  if(e != cudaSuccess || nc < 1) {
    cudaGetLastError();
    *nclusters = 0;
    return GB300_OK;
  }
  if(nc > a.nsys) nc = a.nsys;
  *nclusters = nc;
  cfg.gridDim = dim3((unsigned)(nc * CS), 1, 1);
  if(cudaLaunchKernelEx(&cfg, k_c_solve<T, CS>, a) != cudaSuccess) {
    // a launch the device refuses (nothing ran): the per-kernel form runs
    cudaGetLastError();
    *nclusters = 0;
  }
  return GB300_OK;
}

int gmres_solve_batch_cluster(gb300_matrix *A, const double *val, const double *rhs,
                              double *x, const gb300_solver_params *p, int nsys,
                              const int *off, gb300_solve_info *infos, Work &W,
                              bool *used, const Colouring *mc)
{
  *used = false;
  const int cs = p->batch_kernel;
  if(cs != 1 && cs != 2 && cs != 4 && cs != 8 && cs != 16) return GB300_OK;
  if((p->algorithm != 8 && p->algorithm != 9) ||
     (p->preconditioner != 0 && p->preconditioner != 6))
    return GB300_OK;
  const int m = p->krylov_size <= 1 ? 15 : p->krylov_size;
  // the restart cycles are bounded by the iteration cap inside the kernel
  // (Precision 2, the FP32 factor with FP64 sweeps, takes the per-kernel form)
  if(m > kCMaxKrylov || p->nb_iter_max <= 0 || p->nb_iter_max > 100000000 || nsys < 1 ||
     p->precision == 2)
    return GB300_OK;
  int dev = 0, can = 0;
  GB_CUDA(cudaGetDevice(&dev));
  if(cudaDeviceGetAttribute(&can, cudaDevAttrClusterLaunch, dev) != cudaSuccess || !can) {
    cudaGetLastError();
    return GB300_OK;
  }
  cudaStream_t st = A->ctx->stream;
  const int n = A->n;
  const bool precond = (p->preconditioner == 6);
  const bool fp32 = (p->precision != 0);
  const SysLevels *SL = nullptr;
  // the multicolour order's colour ranges, when A is its permuted copy and
  // they describe the same systems; else the level lists of the schedule
  const bool by_colour = precond && mc && mc->B == A &&
                         (int)mc->seg.size() == nsys + 1 &&
                         std::equal(off, off + nsys + 1, mc->seg.begin()) &&
                         (int)mc->voff.size() == nsys * (mc->ncolors + 1);
  DevBuf<int> dvoff;
  if(precond) {
    if(by_colour) {
      if(mc->ncolors > kCMaxLevels) return GB300_OK;
      GB_TRY(dvoff.alloc(mc->voff.size()));
      GB_CUDA(cudaMemcpyAsync(dvoff.p, mc->voff.data(), sizeof(int) * mc->voff.size(),
                              cudaMemcpyHostToDevice, st));
    }
    else {
      GB_TRY(ilu_sys_levels(A, nsys, off, &SL));
      if(SL->max_levels > kCMaxLevels) return GB300_OK;
    }
    int zr = 0;
    GB_TRY(ilu_factor(A, val, fp32, &zr));
    if(zr) {
      set_error("Zero pivot on line %d in ILU", zr);
      return GB300_ERR_ZERO_PIVOT;
    }
  }
  // the queue: systems by decreasing size (ties by index)
  std::vector<int> order(nsys);
  for(int q = 0; q < nsys; q++) order[q] = q;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    return off[a + 1] - off[a] > off[b + 1] - off[b];
  });
  DevBuf<int> dorder, doff, ints;
  DevBuf<double> dbl;
  GB_TRY(dorder.alloc(nsys));
  GB_TRY(doff.alloc(nsys + 1));
  GB_TRY(ints.alloc(2 * (size_t)nsys + 1));
  GB_TRY(dbl.alloc(3 * (size_t)nsys));
  GB_CUDA(cudaMemcpyAsync(dorder.p, order.data(), sizeof(int) * nsys, cudaMemcpyHostToDevice, st));
  GB_CUDA(cudaMemcpyAsync(doff.p, off, sizeof(int) * (nsys + 1), cudaMemcpyHostToDevice, st));
  GB_CUDA(cudaMemsetAsync(ints.p, 0, sizeof(int) * ints.n, st));
  GB_CUDA(cudaMemsetAsync(dbl.p, 0, sizeof(double) * dbl.n, st));

  const bool flexible = (p->algorithm == 9);
  size_t ldv = (size_t)n;
  double *Vb = (double *)W.vec(0, sizeof(double) * ldv * (m + 1));
  double *Z = flexible ? (double *)W.vec(1, sizeof(double) * ldv * m) : nullptr;
  double *zt = (double *)W.vec(4, sizeof(double) * (n > 0 ? n : 1));
  double *u = (double *)W.vec(3, sizeof(double) * (n > 0 ? n : 1));
  float *t32 = fp32 ? (float *)W.vec(5, sizeof(float) * (n > 0 ? n : 1)) : nullptr;
  if(!Vb || (flexible && !Z) || !zt || !u || (fp32 && !t32)) return GB300_ERR_CUDA;
  GB_CUDA(cudaMemsetAsync(x, 0, sizeof(double) * n, st));

  CArgs a = {};
  a.nsys = nsys;
  a.m = m;
  a.maxit = p->nb_iter_max;
  a.flexible = flexible;
  a.precond = precond;
  a.rtol = p->stopping_test;
  a.order = dorder.p;
  a.off = doff.p;
  a.queue = ints.p + 2 * nsys;
  a.rowptr = A->rowptr.p;
  a.col = A->col.p;
  a.val = val;
  a.rhs = rhs;
  a.x = x;
  if(precond) {
    ilu_factor_arrays(A, fp32, &a.lu, &a.inv, &a.diag);
    if(by_colour) {
      a.ncol = mc->ncolors;
      a.bs = mc->bs;
      a.voff = dvoff.p;
    }
    else {
      a.lrows = SL->lrows.p;
      a.urows = SL->urows.p;
      a.llev = SL->llev.p;
      a.ulev = SL->ulev.p;
      a.llb = SL->llb.p;
      a.ulb = SL->ulb.p;
    }
  }
  a.Vb = Vb;
  a.Z = Z;
  a.zt = zt;
  a.u = u;
  a.t32 = t32;
  a.ldv = ldv;
  a.out_status = ints.p;
  a.out_its = ints.p + nsys;
  a.out_res = dbl.p;
  a.out_rr = dbl.p + nsys;
  a.out_bb = dbl.p + 2 * (size_t)nsys;
  int nc = 0;
  const bool f32 = precond && fp32;
#define GB_LAUNCH_C(CSZ)                                                              \
  GB_TRY(f32 ? launch_c<float, CSZ>(a, st, &nc) : launch_c<double, CSZ>(a, st, &nc))
  switch(cs) {
  case 1: GB_LAUNCH_C(1); break;
  case 2: GB_LAUNCH_C(2); break;
  case 4: GB_LAUNCH_C(4); break;
  case 8: GB_LAUNCH_C(8); break;
  default: GB_LAUNCH_C(16); break;
  }
#undef GB_LAUNCH_C
  // no cluster fits or the launch was refused: nothing ran (x was zeroed, as
  // the per-kernel form does first), and that form solves instead
  if(nc < 1) return GB300_OK;
  std::vector<int> hst(nsys), hits(nsys);
  std::vector<double> hres(nsys), hrr(nsys), hbb(nsys);
  GB_CUDA(cudaMemcpyAsync(hst.data(), a.out_status, sizeof(int) * nsys, cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaMemcpyAsync(hits.data(), a.out_its, sizeof(int) * nsys, cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaMemcpyAsync(hres.data(), a.out_res, sizeof(double) * nsys, cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaMemcpyAsync(hrr.data(), a.out_rr, sizeof(double) * nsys, cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaMemcpyAsync(hbb.data(), a.out_bb, sizeof(double) * nsys, cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  GB_CUDA(cudaGetLastError());
  for(int q = 0; q < nsys; q++) {
    gb300_solve_info &f = infos[q];
    memset(&f, 0, sizeof(f));
    f.status = hst[q];
    f.iterations = hits[q];
    f.residual_estimate = hres[q];
    f.true_residual = sqrt(hrr[q]);
    f.rhs_norm = sqrt(hbb[q]);
    f.ilu_factorized = precond ? 1 : 0;
    f.batch_form = 1;
  }
  *used = true;
  return GB300_OK;
}

}  // namespace gb
