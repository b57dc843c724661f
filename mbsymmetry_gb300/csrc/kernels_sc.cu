// Self-consistent loop kernels (see kernels_sc.h).  The reductions run in
// one CTA with a fixed thread-to-item assignment and a fixed tree, so N and
// the energies are bitwise reproducible from run to run.
#include <algorithm>
#include <cmath>

#include "kernels_sc.h"

namespace gwgb {

namespace {

constexpr int RT = 256;  // threads of the reduction kernels

// Re Tr[A B] for two n x n row-major blocks.
__device__ double re_trace(const double2 *__restrict__ A, const double2 *__restrict__ B, int n) {
  double t = 0.0;
  for (int a = 0; a < n; ++a)
    for (int b = 0; b < n; ++b) {
      const double2 x = A[a * n + b], y = B[b * n + a];
      t += x.x * y.x - x.y * y.y;
    }
  return t;
}

__device__ double block_sum(double v, double *red) {
  red[threadIdx.x] = v;
  __syncthreads();
  for (int s = RT / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  const double r = red[0];
  __syncthreads();
  return r;
}

__global__ void mu_begin_kernel(MuState *st, double *mu_dev, double step) {
  st->mu = st->best_mu;
  st->step = step;
  st->have_lo = st->have_hi = 0;
  st->side = 0;
  st->evals = 0;
  st->done = 0;
  st->best_f = 1e300;
  *mu_dev = st->mu;
}

__global__ void __launch_bounds__(RT) mu_update_kernel(const TrTask *__restrict__ tasks, int ntasks,
                                                       const double2 *__restrict__ Gb,
                                                       const double2 *__restrict__ S, double nscale,
                                                       MuState *st, double *mu_dev, int last) {
  __shared__ double red[RT];
  const bool skip = st->done != 0;
  double part = 0.0;
  if (!skip)
    for (int t = threadIdx.x; t < ntasks; t += RT) {
      const TrTask tk = tasks[t];
      part += tk.w * re_trace(Gb + tk.off, S + tk.off, tk.n);
    }
  const double N = nscale * block_sum(part, red);
  if (threadIdx.x != 0) return;
  if (!skip) {
    const double f = N - st->target;
    st->evals += 1;
    if (!isfinite(f)) {
      st->done = 1;  // a singular Dyson block; the inverse kernel has raised its flag
    } else {
      if (fabs(f) < fabs(st->best_f)) {
        st->best_f = f;
        st->best_mu = st->mu;
      }
      if (fabs(f) <= st->tol) {
        st->done = 1;
      } else {
        const double mu = st->mu;
        int side;
        if (f < 0.0) {
          st->lo = mu; st->flo = f; st->have_lo = 1; side = -1;
        } else {
          st->hi = mu; st->fhi = f; st->have_hi = 1; side = 1;
        }
        double next;
        if (!st->have_hi) {
          next = mu + st->step;
          st->step *= 2.0;
        } else if (!st->have_lo) {
          next = mu - st->step;
          st->step *= 2.0;
        } else {
          // Illinois: the end kept twice in a row has its value halved
          if (side == st->side) {
            if (side < 0) st->fhi *= 0.5; else st->flo *= 0.5;
          }
          st->side = side;
          next = (st->lo * st->fhi - st->hi * st->flo) / (st->fhi - st->flo);
          if (!(next > st->lo && next < st->hi)) next = 0.5 * (st->lo + st->hi);
        }
        st->mu = next;
      }
    }
  }
  if (last || st->done) st->mu = st->best_mu;
  *mu_dev = st->mu;
}

__global__ void mix_kernel(double2 *__restrict__ sig, double2 *__restrict__ sig_old, int64_t n, double alpha) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double2 a = sig[i], b = sig_old[i];
    const double2 v = make_double2(alpha * a.x + (1.0 - alpha) * b.x, alpha * a.y + (1.0 - alpha) * b.y);
    sig[i] = v;
    sig_old[i] = v;
  }
}

__global__ void __launch_bounds__(RT) energy_record_kernel(EnergyArgs a) {
  __shared__ double red[RT];
  double pe = 0.0, po = 0.0, pn = 0.0;
  if (a.with_energy) {
    const int nitem = a.ntasks * a.ncheb;
    for (int it = threadIdx.x; it < nitem; it += RT) {
      const int t = it / a.ncheb, i = it - t * a.ncheb;
      const TrTask tk = a.tasks[t];
      pe += tk.w * re_trace(a.sig + (int64_t)(i + 1) * a.ldt + tk.off, a.hm + (int64_t)i * a.ldt + tk.off, tk.n);
    }
  }
  for (int t = threadIdx.x; t < a.ntasks; t += RT) {
    const TrTask tk = a.tasks[t];
    const double2 *gb = a.g + (int64_t)(a.nts - 1) * a.ldt + tk.off;
    pn += tk.w * re_trace(gb, a.s + tk.off, tk.n);
    if (a.hc) po += tk.w * (re_trace(gb, a.hc + tk.off, tk.n) + re_trace(gb, a.f + tk.off, tk.n));
  }
  const double e = a.ecorr_scale * block_sum(pe, red);
  const double o = a.eone_scale * block_sum(po, red);
  const double N = a.nscale * block_sum(pn, red);
  if (threadIdx.x != 0) return;
  gwgb_sc_record r;
  r.mu = a.st->mu;
  r.n_electrons = N;
  r.e_corr = e;
  r.e_one = o;
  r.leakage = 0.0;
  if (a.leak) {
    const double f = __longlong_as_double((long long)a.leak[0]);
    const double l = __longlong_as_double((long long)a.leak[1]);
    r.leakage = f > 0.0 ? l / f : 0.0;
  }
  r.mu_evals = a.st->evals;
  r.precision = a.precision;
  a.rec[*a.counter] = r;
  *a.counter += 1;
}

}  // namespace

void launch_mu_begin(MuState *st, double *mu_dev, double step, cudaStream_t s) {
  mu_begin_kernel<<<1, 1, 0, s>>>(st, mu_dev, step);
  GWGB_CUDA(cudaGetLastError());
}

void launch_mu_update(const TrTask *tasks, int ntasks, const double2 *Gb, const double2 *S, double nscale,
                      MuState *st, double *mu_dev, int last, cudaStream_t s) {
  mu_update_kernel<<<1, RT, 0, s>>>(tasks, ntasks, Gb, S, nscale, st, mu_dev, last);
  GWGB_CUDA(cudaGetLastError());
}

void launch_mix(double2 *sig, double2 *sig_old, int64_t n, double alpha, cudaStream_t s) {
  if (n == 0) return;
  const int64_t blocks = std::min<int64_t>((n + 255) / 256, 4096);
  mix_kernel<<<(int)blocks, 256, 0, s>>>(sig, sig_old, n, alpha);
  GWGB_CUDA(cudaGetLastError());
}

void launch_energy_record(const EnergyArgs &a, cudaStream_t s) {
  energy_record_kernel<<<1, RT, 0, s>>>(a);
  GWGB_CUDA(cudaGetLastError());
}

}  // namespace gwgb
