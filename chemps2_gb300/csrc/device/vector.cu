// Vector and small dense kernels of the Davidson eigensolver and the truncation step
// (FP64, deterministic reductions).
#include "kernels.cuh"

#include <cmath>

namespace c2g {

namespace {

// ---------------------------------------------------------------- vector kernels

template <int MAXC>
__global__ void __launch_bounds__(kDotThreads) multi_dot_kernel(const double* __restrict__ A, int64_t lda, int ncol,
                                                                const double* __restrict__ x, int64_t n,
                                                                double* __restrict__ partial) {
  double acc[MAXC];
#pragma unroll
  for (int j = 0; j < MAXC; j++) acc[j] = 0.0;
  const int64_t chunk = (n + gridDim.x - 1) / gridDim.x;
  const int64_t start = chunk * blockIdx.x;
  const int64_t end = (start + chunk < n) ? start + chunk : n;
  for (int64_t i = start + threadIdx.x; i < end; i += blockDim.x) {
    const double xi = x[i];
#pragma unroll
    for (int j = 0; j < MAXC; j++)
      if (j < ncol) acc[j] = fma(A[i + lda * j], xi, acc[j]);
  }
  __shared__ double red[kDotThreads / 32][MAXC];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < MAXC; j++) {
    if (j >= ncol) break;
    double v = acc[j];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) red[warp][j] = v;
  }
  __syncthreads();
  if (threadIdx.x < ncol) {
    double v = 0.0;
    for (int w = 0; w < kDotThreads / 32; w++) v += red[w][threadIdx.x];
    partial[static_cast<int64_t>(blockIdx.x) * ncol + threadIdx.x] = v;
  }
}

__global__ void reduce_partials_kernel(const double* __restrict__ partial, int nblk, int ncol, double* __restrict__ out) {
  const int j = threadIdx.x;
  if (j >= ncol) return;
  double v = 0.0;
  for (int b = 0; b < nblk; b++) v += partial[static_cast<int64_t>(b) * ncol + j];
  out[j] = v;
}

__global__ void combine_kernel(double* __restrict__ out, double beta, const double* __restrict__ A, int64_t lda,
                               const double* __restrict__ coef, int ncol, int64_t n) {
  __shared__ double c[64];
  if (threadIdx.x < ncol) c[threadIdx.x] = coef[threadIdx.x];
  __syncthreads();
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    double v = (beta == 0.0) ? 0.0 : beta * out[i];
    for (int j = 0; j < ncol; j++) v = fma(c[j], A[i + lda * j], v);
    out[i] = v;
  }
}

__global__ void scale_kernel(double* x, double s, int64_t n) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    x[i] *= s;
}

__global__ void axpy_kernel(double* y, double a, const double* x, int64_t n) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    y[i] = fma(a, x[i], y[i]);
}

__global__ void fill_kernel(double* x, double v, int64_t n) {
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    x[i] = v;
}

// dst[:, j] = sign_j * src[:, cols - 1 - j], one CTA per column. sign_j makes the entry of
// largest magnitude (the first one on ties) positive, which fixes the gauge of each
// eigenvector so that every executor produces the same singular vectors.
__global__ void reverse_columns_kernel(double* __restrict__ dst, const double* __restrict__ src, int rows, int cols) {
  const int j = blockIdx.x;
  if (j >= cols) return;
  const double* col = src + static_cast<int64_t>(rows) * (cols - 1 - j);
  double best = -1.0;
  int bi = 0;
  for (int i = threadIdx.x; i < rows; i += blockDim.x) {
    const double a = fabs(col[i]);
    if (a > best) {
      best = a;
      bi = i;
    }
  }
  __shared__ double sb[256];
  __shared__ int si[256];
  sb[threadIdx.x] = best;
  si[threadIdx.x] = bi;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      const double b2 = sb[threadIdx.x + o];
      const int i2 = si[threadIdx.x + o];
      if (b2 > sb[threadIdx.x] || (b2 == sb[threadIdx.x] && i2 < si[threadIdx.x])) {
        sb[threadIdx.x] = b2;
        si[threadIdx.x] = i2;
      }
    }
    __syncthreads();
  }
  const double sgn = (col[si[0]] < 0.0) ? -1.0 : 1.0;
  double* out = dst + static_cast<int64_t>(rows) * j;
  for (int i = threadIdx.x; i < rows; i += blockDim.x) out[i] = sgn * col[i];
}

// t -= evals[0] * u   (CheMPS2/Davidson.cpp:280-283)
__global__ void residual_kernel(double* t, const double* u, const double* evals, int64_t n) {
  const double lam = evals[0];
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    t[i] = fma(-lam, u[i], t[i]);
}

__device__ __forceinline__ double precond_den(double d, double cutoff) {
  return (fabs(d) > cutoff) ? d : cutoff;
}

// w = K^-1 u   (CheMPS2/Davidson.cpp:294-305)
__global__ void precond_w_kernel(double* w, const double* u, const double* diag, const double* evals, double cutoff,
                                 int64_t n) {
  const double shift = evals[0];
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    w[i] = u[i] / precond_den(diag[i] - shift, cutoff);
}

// t = -K^-1 (t + alpha u), alpha = -(w.t)/(w.u)   (CheMPS2/Davidson.cpp:306-316)
__global__ void precond_t_kernel(double* t, const double* u, const double* diag, const double* evals,
                                 const double* dots2, double cutoff, int64_t n) {
  const double shift = evals[0];
  const double alpha = -dots2[0] / dots2[1];
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const double v = fma(alpha, u[i], t[i]);
    t[i] = -v / precond_den(diag[i] - shift, cutoff);
  }
}

__global__ void neg_kernel(double* c, int n) {
  if (threadIdx.x < n) c[threadIdx.x] = -c[threadIdx.x];
}

__global__ void inv_sqrt_scale_kernel(double* x, const double* sumsq, int64_t n) {
  const double s = 1.0 / sqrt(sumsq[0]);
  for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x)
    x[i] *= s;
}

__global__ void mxm_row_kernel(double* mxm, int ld, int row, const double* dots, int ncol) {
  const int c = threadIdx.x;
  if (c < ncol) {
    mxm[c + ld * row] = dots[c];
    mxm[row + ld * c] = dots[c];
  }
}

// ---------------------------------------------------------------- small eigenproblems

// Cyclic Jacobi for a symmetric n x n matrix (n <= 32) held in shared memory; one CTA.
// Parallel (round-robin) ordering: every round rotates n/2 disjoint planes at once.
// Eigenvalues ascending in evals[0..n), eigenvectors in the columns of evecs (ld).
constexpr int kEigMax = 32;
struct EigSmem {
  double A[kEigMax][kEigMax + 1];
  double B[kEigMax][kEigMax + 1];
  double Vm[kEigMax][kEigMax + 1];
  double W[kEigMax][kEigMax + 1];
  double cs[kEigMax / 2], sn[kEigMax / 2];
  int pp[kEigMax / 2], qq[kEigMax / 2];
  int role[kEigMax];  // pair index * 2 + (0: p, 1: q), or -1
  int pos[kEigMax];
  double offn, totn;
  int order[kEigMax];
};

// Cyclic Jacobi diagonalisation of the symmetric n x n matrix mat (n <= kEigMax) by one CTA
// (round-robin pairing, n / 2 rotations per round). On return sm.A is diagonal, sm.Vm holds
// the eigenvectors and sm.order lists the eigenvalues in ascending order.
__device__ void jacobi_eig(EigSmem& sm, const double* __restrict__ mat, int n, int ld) {
  double (&A)[kEigMax][kEigMax + 1] = sm.A;
  double (&B)[kEigMax][kEigMax + 1] = sm.B;
  double (&Vm)[kEigMax][kEigMax + 1] = sm.Vm;
  double (&W)[kEigMax][kEigMax + 1] = sm.W;
  double* cs = sm.cs;
  double* sn = sm.sn;
  int* pp = sm.pp;
  int* qq = sm.qq;
  int* role = sm.role;
  int* pos = sm.pos;
  double& offn = sm.offn;
  double& totn = sm.totn;
  int* order = sm.order;
  const int tid = threadIdx.x;
  for (int e = tid; e < n * n; e += blockDim.x) {
    const int i = e % n, j = e / n;
    A[i][j] = mat[i + ld * j];
    Vm[i][j] = (i == j) ? 1.0 : 0.0;
  }
  const int m = (n % 2 == 0) ? n : n + 1;  // padded size; index n is a dummy when odd
  const int npair = m / 2;
  if (tid < m) pos[tid] = tid;
  __syncthreads();
  for (int sweep = 0; sweep < 30; sweep++) {
    if (tid == 0) {
      double off = 0.0, tot = 0.0;
      for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++) {
          const double v = A[i][j] * A[i][j];
          tot += v;
          if (i != j) off += v;
        }
      offn = off;
      totn = tot;
    }
    __syncthreads();
    if (!(offn > 1e-28 * totn) || n < 2) break;
    for (int round = 0; round < m - 1; round++) {
      if (tid < m) role[tid] = -1;
      __syncthreads();
      if (tid < npair) {
        int p = pos[tid], q = pos[m - 1 - tid];
        if (p > q) { const int t = p; p = q; q = t; }
        double c = 1.0, s = 0.0;
        if (q < n) {
          const double apq = A[p][q];
          if (apq != 0.0) {
            const double tau = (A[q][q] - A[p][p]) / (2.0 * apq);
            const double t = (tau >= 0.0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
            c = 1.0 / sqrt(1.0 + t * t);
            s = t * c;
          }
          role[p] = 2 * tid;
          role[q] = 2 * tid + 1;
        }
        cs[tid] = c;
        sn[tid] = s;
        pp[tid] = p;
        qq[tid] = q;
      }
      __syncthreads();
      // rows: B = J^T A
      for (int e = tid; e < n * n; e += blockDim.x) {
        const int i = e % n, j = e / n;
        const int r = role[i];
        double v = A[i][j];
        if (r >= 0) {
          const int k = r >> 1;
          const double c = cs[k], s = sn[k];
          v = (r & 1) ? s * A[pp[k]][j] + c * A[qq[k]][j] : c * A[pp[k]][j] - s * A[qq[k]][j];
        }
        B[i][j] = v;
      }
      __syncthreads();
      // columns: A = B J, V = V J
      for (int e = tid; e < n * n; e += blockDim.x) {
        const int i = e % n, j = e / n;
        const int r = role[j];
        double v = B[i][j], w = Vm[i][j];
        if (r >= 0) {
          const int k = r >> 1;
          const double c = cs[k], s = sn[k];
          if (r & 1) {
            v = s * B[i][pp[k]] + c * B[i][qq[k]];
            w = s * Vm[i][pp[k]] + c * Vm[i][qq[k]];
          } else {
            v = c * B[i][pp[k]] - s * B[i][qq[k]];
            w = c * Vm[i][pp[k]] - s * Vm[i][qq[k]];
          }
        }
        A[i][j] = v;
        W[i][j] = w;
      }
      __syncthreads();
      for (int e = tid; e < n * n; e += blockDim.x) {
        const int i = e % n, j = e / n;
        Vm[i][j] = W[i][j];
      }
      // next pairing: position 0 fixed, the others rotate
      if (tid == 0) {
        const int last = pos[m - 1];
        for (int k = m - 1; k > 1; k--) pos[k] = pos[k - 1];
        pos[1] = last;
      }
      __syncthreads();
    }
  }
  if (tid == 0) {
    for (int i = 0; i < n; i++) order[i] = i;
    for (int i = 0; i < n; i++) {  // selection sort, ascending
      int best = i;
      for (int j = i + 1; j < n; j++)
        if (A[order[j]][order[j]] < A[order[best]][order[best]]) best = j;
      const int t = order[i];
      order[i] = order[best];
      order[best] = t;
    }
  }
  __syncthreads();
}

// The Rayleigh-Ritz eigenproblem of the Davidson solver (CheMPS2/Davidson.cpp:242-276,
// where the reference calls dsyev on the <= 32 x 32 projected matrix): cyclic Jacobi with
// the round-robin (Brent-Luk) ordering, n / 2 disjoint rotations per round, one thread per
// matrix element. A round is two barriers: the pair leaders compute their rotations, then
// every thread forms its element of J^T A J and of V J from the four (two) elements it
// depends on, into the other buffer. The pairs of round r are fixed by position:
// pos(0) = 0, pos(k) = 1 + (k - 1 - r mod m - 1), pairs (pos(t), pos(m - 1 - t)).
// Warm start (Davidson expansion): the matrix grew by one row and column since the
// previous call, whose eigenvectors E are still in evecs; the solver starts from
// A = diag(E, 1)^T M diag(E, 1) (diagonal but for the last row and column) and V = diag(E, 1),
// which takes two to three sweeps instead of six to ten.
constexpr int kRrThreads = kEigMax * kEigMax;
__global__ void __launch_bounds__(kRrThreads) rr_eig_kernel(const double* __restrict__ mat, int n, int ld,
                                                            double* __restrict__ evals, double* __restrict__ evecs,
                                                            int warm) {
  __shared__ double A[2][kEigMax][kEigMax + 1];
  __shared__ double V[2][kEigMax][kEigMax + 1];
  __shared__ double alpha[kEigMax], beta[kEigMax];
  __shared__ int partner[kEigMax];
  __shared__ double red[2][kEigMax];
  __shared__ int done;
  __shared__ int rank[kEigMax];
  const int tid = threadIdx.x;
  const int i = tid % kEigMax, j = tid / kEigMax;  // element (i, j), column-major
  const bool in = i < n && j < n;
  // ---- start
  if (warm) {
    // E (n - 1 columns of the previous call, ld) extended by the unit vector e_{n-1}
    auto Ehat = [&](int a, int b) -> double {
      if (a == n - 1 || b == n - 1) return (a == b) ? 1.0 : 0.0;
      return evecs[a + ld * b];
    };
    double t = 0.0;  // T = M Ehat, element (i, j)
    if (in)
      for (int b = 0; b < n; b++) t = fma(mat[i + ld * b], Ehat(b, j), t);
    A[1][i][j] = t;
    V[0][i][j] = in ? Ehat(i, j) : 0.0;
    __syncthreads();
    double g = 0.0;  // Ehat^T T
    if (in)
      for (int a = 0; a < n; a++) g = fma(V[0][a][i], A[1][a][j], g);
    A[0][i][j] = g;
  } else {
    A[0][i][j] = in ? mat[i + ld * j] : 0.0;
    V[0][i][j] = (in && i == j) ? 1.0 : 0.0;
  }
  __syncthreads();
  {  // exact symmetry of the starting matrix
    const double a = in ? 0.5 * (A[0][i][j] + A[0][j][i]) : 0.0;
    __syncthreads();
    if (in) A[0][i][j] = a;
  }
  __syncthreads();
  const int m = (n % 2 == 0) ? n : n + 1;  // index n is a dummy when n is odd
  const int npair = m / 2;
  int cur = 0;
  for (int sweep = 0; sweep < 30 && n > 1; sweep++) {
    // convergence: off-diagonal against total squared norm (every thread takes one element)
    {
      const double v = in ? A[cur][i][j] * A[cur][i][j] : 0.0;
      double off = (i != j) ? v : 0.0, tot = v;
      for (int o = 16; o > 0; o >>= 1) {
        off += __shfl_down_sync(0xffffffffu, off, o);
        tot += __shfl_down_sync(0xffffffffu, tot, o);
      }
      if ((tid & 31) == 0) {
        red[0][tid >> 5] = off;
        red[1][tid >> 5] = tot;
      }
      __syncthreads();
      if (tid == 0) {
        double so = 0.0, st = 0.0;
        for (int w = 0; w < kEigMax; w++) {
          so += red[0][w];
          st += red[1][w];
        }
        done = !(so > 1e-28 * st);
      }
      __syncthreads();
      if (done) break;
    }
    for (int r = 0; r < m - 1; r++) {
      if (tid < npair) {
        const int k1 = tid, k2 = m - 1 - tid;
        const int a = (k1 == 0) ? 0 : 1 + ((k1 - 1 - r) % (m - 1) + (m - 1)) % (m - 1);
        const int b = 1 + ((k2 - 1 - r) % (m - 1) + (m - 1)) % (m - 1);
        const int p = a < b ? a : b, q = a < b ? b : a;
        double c = 1.0, s = 0.0;
        if (q < n) {
          const double apq = A[cur][p][q];
          if (apq != 0.0) {
            const double tau = (A[cur][q][q] - A[cur][p][p]) / (2.0 * apq);
            const double t = (tau >= 0.0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
            c = 1.0 / sqrt(1.0 + t * t);
            s = t * c;
          }
          partner[p] = q;
          partner[q] = p;
          alpha[p] = c;
          beta[p] = -s;
          alpha[q] = c;
          beta[q] = s;
        } else if (p < n) {  // paired with the dummy: untouched
          partner[p] = p;
          alpha[p] = 1.0;
          beta[p] = 0.0;
        }
      }
      __syncthreads();
      const int nxt = cur ^ 1;
      if (in) {
        const int pi = partner[i], pj = partner[j];
        const double ai = alpha[i], bi = beta[i], aj = alpha[j], bj = beta[j];
        // B = J^T A rows i: ai A[i] + bi A[pi]; then columns j: aj B[.][j] + bj B[.][pj]
        const double bij = ai * A[cur][i][j] + bi * A[cur][pi][j];
        const double bipj = ai * A[cur][i][pj] + bi * A[cur][pi][pj];
        A[nxt][i][j] = aj * bij + bj * bipj;
        V[nxt][i][j] = aj * V[cur][i][j] + bj * V[cur][i][pj];
      }
      cur = nxt;
      __syncthreads();
    }
  }
  // ascending order: the rank of each eigenvalue (ties by index)
  if (tid < n) {
    const double lam = A[cur][tid][tid];
    int rk = 0;
    for (int k = 0; k < n; k++) {
      const double o = A[cur][k][k];
      rk += (o < lam || (o == lam && k < tid)) ? 1 : 0;
    }
    rank[tid] = rk;
    evals[rk] = lam;
  }
  __syncthreads();
  if (in) evecs[i + ld * rank[j]] = V[cur][i][j];
}

// One CTA per job: Jacobi eigendecomposition of the n x n Gram matrix at base + offG; the
// eigenvalues go to base + offE in ascending order and the eigenvectors to base + offU in
// descending order of the eigenvalue, each with the sign that makes its largest-magnitude
// entry (the first one on ties) positive -- the layout launch_reverse_columns produces.
__global__ void __launch_bounds__(256) batched_eig_kernel(const EigJob* __restrict__ jobs, double* __restrict__ base) {
  __shared__ EigSmem sm;
  __shared__ double sgn[kEigMax];
  const EigJob jb = jobs[blockIdx.x];
  const int n = jb.n;
  jacobi_eig(sm, base + jb.offG, n, n);
  const int tid = threadIdx.x;
  if (tid < n) {
    base[jb.offE + tid] = sm.A[sm.order[tid]][sm.order[tid]];
    const int col = sm.order[n - 1 - tid];  // output column tid
    double best = -1.0, v = 0.0;
    for (int i = 0; i < n; i++) {
      const double a = fabs(sm.Vm[i][col]);
      if (a > best) {
        best = a;
        v = sm.Vm[i][col];
      }
    }
    sgn[tid] = (v < 0.0) ? -1.0 : 1.0;
  }
  __syncthreads();
  for (int e = tid; e < n * n; e += blockDim.x) {
    const int i = e % n, j = e / n;
    base[jb.offU + i + static_cast<int64_t>(n) * j] = sgn[j] * sm.Vm[i][sm.order[n - 1 - j]];
  }
}

// Loewdin orthonormaliser of k <= 4 vectors: L = S^-1/2 from the k x k overlap S
// (CheMPS2/Davidson.cpp:367-381). Serial Jacobi, one thread.
__global__ void lowdin_kernel(const double* __restrict__ overlap, int k, double* __restrict__ lowdin) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double a[4][4], v[4][4];
  for (int i = 0; i < k; i++)
    for (int j = 0; j < k; j++) {
      a[i][j] = overlap[i + k * j];
      v[i][j] = (i == j) ? 1.0 : 0.0;
    }
  for (int sweep = 0; sweep < 50; sweep++) {
    double off = 0.0;
    for (int i = 0; i < k; i++)
      for (int j = 0; j < k; j++)
        if (i != j) off += a[i][j] * a[i][j];
    if (off < 1e-60) break;
    for (int p = 0; p < k; p++)
      for (int q = p + 1; q < k; q++) {
        if (a[p][q] == 0.0) continue;
        const double tau = (a[q][q] - a[p][p]) / (2.0 * a[p][q]);
        const double t = (tau >= 0.0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
        const double c = 1.0 / sqrt(1.0 + t * t), s = t * c;
        for (int j = 0; j < k; j++) {
          const double x = a[p][j], y = a[q][j];
          a[p][j] = c * x - s * y;
          a[q][j] = s * x + c * y;
        }
        for (int i = 0; i < k; i++) {
          const double x = a[i][p], y = a[i][q];
          a[i][p] = c * x - s * y;
          a[i][q] = s * x + c * y;
          const double vx = v[i][p], vy = v[i][q];
          v[i][p] = c * vx - s * vy;
          v[i][q] = s * vx + c * vy;
        }
      }
  }
  double f[4];
  for (int j = 0; j < k; j++) f[j] = pow(a[j][j], -0.5);
  for (int i = 0; i < k; i++)
    for (int j = 0; j < k; j++) {
      double s = 0.0;
      for (int l = 0; l < k; l++) s += v[i][l] * f[l] * v[j][l];
      lowdin[i + k * j] = s;
    }
}

inline int grid_for(int64_t n, int threads = 256) {
  int64_t b = (n + threads - 1) / threads;
  if (b > 152 * 8) b = 152 * 8;
  if (b < 1) b = 1;
  return static_cast<int>(b);
}

}  // namespace

cudaError_t launch_multi_dot(const double* A, int64_t lda, int ncol, const double* x, int64_t n, double* partial,
                             double* out, cudaStream_t stream) {
  if (ncol <= 0) return cudaSuccess;
  if (ncol > 32) return cudaErrorInvalidValue;
  if (ncol <= 4)
    multi_dot_kernel<4><<<kDotBlocks, kDotThreads, 0, stream>>>(A, lda, ncol, x, n, partial);
  else if (ncol <= 8)
    multi_dot_kernel<8><<<kDotBlocks, kDotThreads, 0, stream>>>(A, lda, ncol, x, n, partial);
  else
    multi_dot_kernel<32><<<kDotBlocks, kDotThreads, 0, stream>>>(A, lda, ncol, x, n, partial);
  reduce_partials_kernel<<<1, 32, 0, stream>>>(partial, kDotBlocks, ncol, out);
  return cudaGetLastError();
}

cudaError_t launch_combine(double* out, double beta, const double* A, int64_t lda, const double* coef, int ncol,
                           int64_t n, cudaStream_t stream) {
  if (ncol > 64) return cudaErrorInvalidValue;
  if (n <= 0) return cudaSuccess;
  combine_kernel<<<grid_for(n), 256, 0, stream>>>(out, beta, A, lda, coef, ncol, n);
  return cudaGetLastError();
}

cudaError_t launch_norm2(const double* x, int64_t n, double* partial, double* out, cudaStream_t stream) {
  return launch_multi_dot(x, n, 1, x, n, partial, out, stream);
}

cudaError_t launch_scale(double* x, double s, int64_t n, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  scale_kernel<<<grid_for(n), 256, 0, stream>>>(x, s, n);
  return cudaGetLastError();
}

cudaError_t launch_axpy(double* y, double a, const double* x, int64_t n, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  axpy_kernel<<<grid_for(n), 256, 0, stream>>>(y, a, x, n);
  return cudaGetLastError();
}

cudaError_t launch_fill(double* x, double v, int64_t n, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  fill_kernel<<<grid_for(n), 256, 0, stream>>>(x, v, n);
  return cudaGetLastError();
}

cudaError_t launch_reverse_columns(double* dst, const double* src, int rows, int cols, cudaStream_t stream) {
  if (rows <= 0 || cols <= 0) return cudaSuccess;
  reverse_columns_kernel<<<cols, 256, 0, stream>>>(dst, src, rows, cols);
  return cudaGetLastError();
}

cudaError_t launch_small_eig(double* mat, int n, int ld, double* evals, double* evecs, cudaStream_t stream,
                             bool warm) {
  if (n < 1 || n > kEigMax || ld < n) return cudaErrorInvalidValue;
  rr_eig_kernel<<<1, kRrThreads, 0, stream>>>(mat, n, ld, evals, evecs, warm && n > 1 ? 1 : 0);
  return cudaGetLastError();
}

// Cyclic Jacobi as in jacobi_eig, for kBatchedEigMax < n <= kBatchedEigLargeMax: the
// matrix A (n x (n + 1), padded rows) lives in dynamic shared memory; each round's n / 2
// disjoint plane rotations update the rows p, q and then the columns p, q of A in place,
// and the same columns of the eigenvector matrix V, which is kept in global memory at the
// job's Gram slot (read into A first). Output as batched_eig_kernel: eigenvalues ascending
// at offE, eigenvectors in descending order of the eigenvalue with the sign gauge at offU.
constexpr int kEigLargeThreads = 512;
struct EigLargeShared {
  double cs[kBatchedEigLargeMax / 2], sn[kBatchedEigLargeMax / 2];
  int pp[kBatchedEigLargeMax / 2], qq[kBatchedEigLargeMax / 2];
  int pos[kBatchedEigLargeMax];
  int order[kBatchedEigLargeMax];
  double sgn[kBatchedEigLargeMax];
  double red[2][kEigLargeThreads / 32];
};

__global__ void __launch_bounds__(kEigLargeThreads) batched_eig_large_kernel(const EigJob* __restrict__ jobs,
                                                                             double* __restrict__ base) {
  extern __shared__ double dyn[];
  __shared__ EigLargeShared sh;
  const EigJob jb = jobs[blockIdx.x];
  const int n = jb.n, ldA = n + 1;
  double* A = dyn;                  // A[i + ldA j] is element (i, j)... stored row-major: A[i * ldA + j]
  double* V = base + jb.offG;       // V(i, j) = V[i + n j]
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int e = tid; e < n * n; e += nt) {
    const int i = e % n, j = e / n;
    A[i * ldA + j] = V[i + static_cast<int64_t>(n) * j];
  }
  __syncthreads();
  for (int e = tid; e < n * n; e += nt) {
    const int i = e % n, j = e / n;
    V[i + static_cast<int64_t>(n) * j] = (i == j) ? 1.0 : 0.0;
  }
  const int m = (n % 2 == 0) ? n : n + 1;
  const int npair = m / 2;
  if (tid < m) sh.pos[tid] = tid;
  __syncthreads();
  for (int sweep = 0; sweep < 30; sweep++) {
    double off = 0.0, tot = 0.0;
    for (int e = tid; e < n * n; e += nt) {
      const int i = e % n, j = e / n;
      const double v = A[i * ldA + j] * A[i * ldA + j];
      tot += v;
      if (i != j) off += v;
    }
    for (int o = 16; o > 0; o >>= 1) {
      off += __shfl_down_sync(0xffffffffu, off, o);
      tot += __shfl_down_sync(0xffffffffu, tot, o);
    }
    if ((tid & 31) == 0) {
      sh.red[0][tid >> 5] = off;
      sh.red[1][tid >> 5] = tot;
    }
    __syncthreads();
    off = 0.0;
    tot = 0.0;
    for (int w = 0; w < nt / 32; w++) {
      off += sh.red[0][w];
      tot += sh.red[1][w];
    }
    __syncthreads();
    if (!(off > 1e-28 * tot)) break;
    for (int round = 0; round < m - 1; round++) {
      if (tid < npair) {
        int p = sh.pos[tid], q = sh.pos[m - 1 - tid];
        if (p > q) {
          const int t = p;
          p = q;
          q = t;
        }
        double c = 1.0, s = 0.0;
        if (q < n) {
          const double apq = A[p * ldA + q];
          if (apq != 0.0) {
            const double tau = (A[q * ldA + q] - A[p * ldA + p]) / (2.0 * apq);
            const double t = (tau >= 0.0 ? 1.0 : -1.0) / (fabs(tau) + sqrt(1.0 + tau * tau));
            c = 1.0 / sqrt(1.0 + t * t);
            s = t * c;
          }
        } else {
          q = p;  // the dummy plane of an odd n: no rotation
        }
        sh.cs[tid] = c;
        sh.sn[tid] = s;
        sh.pp[tid] = p;
        sh.qq[tid] = q;
      }
      __syncthreads();
      // rows p, q of every plane: A <- J^T A
      for (int e = tid; e < npair * n; e += nt) {
        const int k = e / n, j = e % n;
        const int p = sh.pp[k], q = sh.qq[k];
        if (p == q) continue;
        const double c = sh.cs[k], s = sh.sn[k];
        const double a = A[p * ldA + j], b = A[q * ldA + j];
        A[p * ldA + j] = c * a - s * b;
        A[q * ldA + j] = s * a + c * b;
      }
      __syncthreads();
      // columns p, q: A <- A J, V <- V J
      for (int e = tid; e < npair * n; e += nt) {
        const int k = e / n, i = e % n;
        const int p = sh.pp[k], q = sh.qq[k];
        if (p == q) continue;
        const double c = sh.cs[k], s = sh.sn[k];
        const double a = A[i * ldA + p], b = A[i * ldA + q];
        A[i * ldA + p] = c * a - s * b;
        A[i * ldA + q] = s * a + c * b;
        double* vp = V + static_cast<int64_t>(n) * p;
        double* vq = V + static_cast<int64_t>(n) * q;
        const double x = vp[i], y = vq[i];
        vp[i] = c * x - s * y;
        vq[i] = s * x + c * y;
      }
      __syncthreads();
      if (tid == 0) {
        const int last = sh.pos[m - 1];
        for (int k = m - 1; k > 1; k--) sh.pos[k] = sh.pos[k - 1];
        sh.pos[1] = last;
      }
      __syncthreads();
    }
  }
  if (tid == 0) {
    for (int i = 0; i < n; i++) sh.order[i] = i;
    for (int i = 0; i < n; i++) {  // selection sort, ascending
      int best = i;
      for (int j = i + 1; j < n; j++)
        if (A[sh.order[j] * ldA + sh.order[j]] < A[sh.order[best] * ldA + sh.order[best]]) best = j;
      const int t = sh.order[i];
      sh.order[i] = sh.order[best];
      sh.order[best] = t;
    }
  }
  __syncthreads();
  if (tid < n) {
    base[jb.offE + tid] = A[sh.order[tid] * ldA + sh.order[tid]];
    const double* col = V + static_cast<int64_t>(n) * sh.order[n - 1 - tid];  // output column tid
    double best = -1.0, v = 0.0;
    for (int i = 0; i < n; i++) {
      const double a = fabs(col[i]);
      if (a > best) {
        best = a;
        v = col[i];
      }
    }
    sh.sgn[tid] = (v < 0.0) ? -1.0 : 1.0;
  }
  __syncthreads();
  for (int e = tid; e < n * n; e += nt) {
    const int i = e % n, j = e / n;
    base[jb.offU + i + static_cast<int64_t>(n) * j] = sh.sgn[j] * V[i + static_cast<int64_t>(n) * sh.order[n - 1 - j]];
  }
}

cudaError_t launch_batched_eig_large(const EigJob* jobs, int njobs, int nmax, double* base, cudaStream_t stream) {
  if (njobs <= 0) return cudaSuccess;
  if (nmax > kBatchedEigLargeMax) return cudaErrorInvalidValue;
  const size_t bytes = sizeof(double) * static_cast<size_t>(nmax) * (nmax + 1);
  cudaError_t e = cudaFuncSetAttribute(batched_eig_large_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(bytes));
  if (e != cudaSuccess) return e;
  batched_eig_large_kernel<<<njobs, kEigLargeThreads, bytes, stream>>>(jobs, base);
  return cudaGetLastError();
}

cudaError_t launch_batched_eig(const EigJob* jobs, int njobs, double* base, cudaStream_t stream) {
  if (njobs <= 0) return cudaSuccess;
  batched_eig_kernel<<<njobs, 256, 0, stream>>>(jobs, base);
  return cudaGetLastError();
}

cudaError_t launch_residual(double* t, const double* u, const double* evals, int64_t n, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  residual_kernel<<<grid_for(n), 256, 0, stream>>>(t, u, evals, n);
  return cudaGetLastError();
}

cudaError_t launch_precond_w(double* w, const double* u, const double* diag, const double* evals, double cutoff,
                             int64_t n, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  precond_w_kernel<<<grid_for(n), 256, 0, stream>>>(w, u, diag, evals, cutoff, n);
  return cudaGetLastError();
}

cudaError_t launch_precond_t(double* t, const double* u, const double* diag, const double* evals,
                             const double* dots2, double cutoff, int64_t n, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  precond_t_kernel<<<grid_for(n), 256, 0, stream>>>(t, u, diag, evals, dots2, cutoff, n);
  return cudaGetLastError();
}

cudaError_t launch_neg(double* c, int n, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  neg_kernel<<<1, 64, 0, stream>>>(c, n);
  return cudaGetLastError();
}

cudaError_t launch_inv_sqrt_scale(double* x, const double* sumsq, int64_t n, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  inv_sqrt_scale_kernel<<<grid_for(n), 256, 0, stream>>>(x, sumsq, n);
  return cudaGetLastError();
}

cudaError_t launch_mxm_row(double* mxm, int ld, int row, const double* dots, int ncol, cudaStream_t stream) {
  mxm_row_kernel<<<1, 64, 0, stream>>>(mxm, ld, row, dots, ncol);
  return cudaGetLastError();
}

cudaError_t launch_lowdin(const double* overlap, int k, double* lowdin, cudaStream_t stream) {
  if (k < 1 || k > 4) return cudaErrorInvalidValue;
  lowdin_kernel<<<1, 32, 0, stream>>>(overlap, k, lowdin);
  return cudaGetLastError();
}

}  // namespace c2g
