// SPAI-1 on the matrix's own pattern (Preconditioner 25): for each row i,
// g_i = argmin || e_i - A g ||_2 over the vectors supported on row i's
// columns J, the least-squares sparse approximate inverse of Grote and
// Huckle restricted to A's pattern.  For a symmetric A the normal
// equations are (A^2)_JJ g = A_Ji: (A^2)_jk is the dot product of rows j
// and k (a merge of two sorted rows), and the system (|J| <= 16 unknowns)
// is solved by Cholesky, one thread per row.  The rows g_i^T form G with
// G A ~ I, the smoother z = G v of the two-level cycle.  No counterpart in
// Sparskit.
#include "common.cuh"
#include "krylov.cuh"

namespace gb {

constexpr int kSpaiMax = 16;

__global__ void k_spai1(int n, const int *__restrict__ rowptr, const int *__restrict__ col,
                        const double *__restrict__ val, double *__restrict__ G, int *err)
{
  for(int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int s = rowptr[i], m = rowptr[i + 1] - s;
    if(m < 1 || m > kSpaiMax) {
      atomicCAS(err, 0, i + 1);
      for(int a = 0; a < m; a++) G[s + a] = 0.;
      continue;
    }
    double N[kSpaiMax * (kSpaiMax + 1) / 2], r[kSpaiMax];
    for(int a = 0; a < m; a++) {
      const int j = col[s + a];
      const int sj = rowptr[j], ej = rowptr[j + 1];
      const int pij = find_col(col, sj, ej, i);
      r[a] = pij >= 0 ? val[pij] : 0.;
      for(int b = 0; b <= a; b++) {
        const int k = col[s + b];
        int p = sj, q = rowptr[k];
        const int eq = rowptr[k + 1];
        double d = 0.;
        while(p < ej && q < eq) {
          const int cp = col[p], cq = col[q];
          if(cp == cq) {
            d = fma(val[p], val[q], d);
            p++;
            q++;
          }
          else if(cp < cq)
            p++;
          else
            q++;
        }
        N[a * (a + 1) / 2 + b] = d;
      }
    }
    // Cholesky of the packed lower triangle, in place
    bool ok = true;
    for(int a = 0; a < m && ok; a++) {
      for(int b = 0; b <= a; b++) {
        double t = N[a * (a + 1) / 2 + b];
        for(int c = 0; c < b; c++) t -= N[a * (a + 1) / 2 + c] * N[b * (b + 1) / 2 + c];
        if(a == b) {
          if(!(t > 0.)) {
            ok = false;
            break;
          }
          N[a * (a + 1) / 2 + a] = sqrt(t);
        }
        else
          N[a * (a + 1) / 2 + b] = t / N[b * (b + 1) / 2 + b];
      }
    }
    if(!ok) {
      atomicCAS(err, 0, i + 1);
      for(int a = 0; a < m; a++) G[s + a] = 0.;
      continue;
    }
    for(int a = 0; a < m; a++) {  // L y = r
      double t = r[a];
      for(int c = 0; c < a; c++) t -= N[a * (a + 1) / 2 + c] * r[c];
      r[a] = t / N[a * (a + 1) / 2 + a];
    }
    for(int a = m - 1; a >= 0; a--) {  // L^T g = y
      double t = r[a];
      for(int c = a + 1; c < m; c++) t -= N[c * (c + 1) / 2 + a] * r[c];
      r[a] = t / N[a * (a + 1) / 2 + a];
    }
    for(int a = 0; a < m; a++) G[s + a] = r[a];
  }
}

int spai1(gb300_matrix *A, const double *val)
{
  cudaStream_t st = A->ctx->stream;
  GB_TRY(A->corr.alloc(A->nnz));
  DevBuf<int> err;
  GB_TRY(err.alloc(1));
  GB_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), st));
  k_spai1<<<grid_for(A->n, 128, 152 * 64), 128, 0, st>>>(A->n, A->rowptr.p, A->col.p, val,
                                                          A->corr.p, err.p);
  GB_CUDA(cudaGetLastError());
  int e = 0;
  GB_CUDA(cudaMemcpyAsync(&e, err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  GB_CUDA(cudaStreamSynchronize(st));
  if(e) {
    set_error("SPAI-1: row %d has more than %d entries or singular normal equations "
              "(Preconditioner 25 wants a symmetric matrix with short rows)", e - 1, kSpaiMax);
    return GB300_ERR_UNSUPPORTED;
  }
  A->corr_version = A->pattern_version;
  return GB300_OK;
}

}  // namespace gb
