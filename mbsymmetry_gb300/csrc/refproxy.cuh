// Reference-GPU proxy: the reference's cuBLAS call sequence for the two
// contractions of one GW iteration, replayed on this GPU for measurement
// (gwgb_refproxy_run).  It is not on the drop-in path: the engine's own
// kernels never call it, and cuBLAS is loaded (dlopen) only when it runs.
//
// Call sequence, per SymmetryMBPT/src/cuda (file:line):
//   G rotation, cugw_routines_block.cu:164-184: per rotated block two
//     ZGEMM_SB over nts*ns (O X, then (O X) O^H) and a DSCAL of the imaginary
//     parts for a time-reversal partner; slice copies otherwise;
//   G(-tau), cugw_routines_block.cu:189-199: one D2D copy per (k, tau);
//   P0, cugw_qkpt_block.cu:119-130, 195-284, per (q_irr, k) pair on stream
//     pair % nstreams: GEAM transpose per V block (V_Qpm -> V_pmQ), a
//     conjugated copy of the pair's V (DSCAL), then per tau batch and spin a
//     memset of the pair-local P0 and per V block three ZGEMM_SB
//       X1 = G(beta - tau) V_pmQ, X2 = conj(V) G(tau)^T, P0 += c X2 X1,
//     and one ZAXPY of the local P0 into the accumulator;
//   Sigma, cugw_qkpt_block.cu:140-192, 288-436, per (k_irr, q) pair: P~(q)
//     from P~(q_irr) (per auxrep block two ZGEMM_SB over nts and a DSCAL, or a
//     D2D copy), GEAM conj-transpose per V block (V_Qim -> V_nPj), per tau
//     batch and spin per V block three ZGEMM_SB
//       Y1 = V G(tau), Y2 = Y1 P~(tau), Sigma -= Y2 V_nPj,
//     and one ZAXPY of the pair-local Sigma per pair.
// Two differences, both in the reference's favour: V stays in HBM (the
// reference copies each pair's V slice from a host window,
// cugw_qkpt_block.cu:78-137), and the device locks that serialise the
// accumulation (cugw_qkpt_block.cu:271-284, 417-435) become one accumulator
// per stream, summed at the end.

#include <cublas_v2.h>
#include <dlfcn.h>

namespace gwgb {
namespace {

struct CublasApi {
  decltype(&cublasCreate_v2) create = nullptr;
  decltype(&cublasDestroy_v2) destroy = nullptr;
  decltype(&cublasSetStream_v2) set_stream = nullptr;
  decltype(&cublasZgemmStridedBatched) zgemm_sb = nullptr;
  decltype(&cublasZgeam) zgeam = nullptr;
  decltype(&cublasDscal_v2) dscal = nullptr;
  decltype(&cublasZaxpy_v2) zaxpy = nullptr;
  decltype(&cublasZdscal_v2) zdscal = nullptr;
  bool ok = false;
};

const CublasApi &cublas_api() {
  static CublasApi api = [] {
    CublasApi a;
    void *h = nullptr;
    for (const char *n : {"libcublas.so.13", "/usr/local/cuda/lib64/libcublas.so.13", "libcublas.so"})
      if ((h = dlopen(n, RTLD_NOW | RTLD_LOCAL)) != nullptr) break;
    if (!h) return a;
    a.create = (decltype(a.create))dlsym(h, "cublasCreate_v2");
    a.destroy = (decltype(a.destroy))dlsym(h, "cublasDestroy_v2");
    a.set_stream = (decltype(a.set_stream))dlsym(h, "cublasSetStream_v2");
    a.zgemm_sb = (decltype(a.zgemm_sb))dlsym(h, "cublasZgemmStridedBatched");
    a.zgeam = (decltype(a.zgeam))dlsym(h, "cublasZgeam");
    a.dscal = (decltype(a.dscal))dlsym(h, "cublasDscal_v2");
    a.zaxpy = (decltype(a.zaxpy))dlsym(h, "cublasZaxpy_v2");
    a.zdscal = (decltype(a.zdscal))dlsym(h, "cublasZdscal_v2");
    a.ok = a.create && a.destroy && a.set_stream && a.zgemm_sb && a.zgeam && a.dscal && a.zaxpy && a.zdscal;
    return a;
  }();
  return api;
}

#define GWGB_CUBLAS(x)                                                                     \
  do {                                                                                     \
    const cublasStatus_t s_ = (x);                                                         \
    if (s_ != CUBLAS_STATUS_SUCCESS)                                                       \
      throw ::gwgb::Error(GWGB_E_CUDA, std::string("cuBLAS call failed (status ") +            \
                                       std::to_string((int)s_) + "): " #x);                \
  } while (0)

// Streams, events and the cuBLAS handle of one proxy run, released on every exit.
struct ProxyResources {
  const CublasApi &cb;
  cublasHandle_t h = nullptr;
  std::vector<cudaStream_t> ss;
  std::vector<cudaEvent_t> ev;
  explicit ProxyResources(const CublasApi &api) : cb(api) {}
  ~ProxyResources() {
    if (h) cb.destroy(h);
    for (cudaStream_t s : ss)
      if (s) cudaStreamDestroy(s);
    for (cudaEvent_t e : ev)
      if (e) cudaEventDestroy(e);
  }
  cudaEvent_t event(unsigned flags) {
    cudaEvent_t e = nullptr;
    GWGB_CUDA(cudaEventCreateWithFlags(&e, flags));
    ev.push_back(e);
    return e;
  }
};

inline cuDoubleComplex cz(double re, double im = 0.0) { return make_cuDoubleComplex(re, im); }
inline cuDoubleComplex *zc(double2 *p) { return reinterpret_cast<cuDoubleComplex *>(p); }
inline const cuDoubleComplex *zc(const double2 *p) { return reinterpret_cast<const cuDoubleComplex *>(p); }

}  // namespace

void Engine::refproxy(int nt_batch, int nstreams, gwgb_proxy_stats *out) {
  GWGB_REQUIRE(have_V_, GWGB_E_STATE, "V has not been uploaded");
  GWGB_REQUIRE(nt_batch >= 1 && nt_batch <= nts_ && nstreams >= 1 && nstreams <= 64, GWGB_E_INVALID,
               "nt_batch must be in [1, nts] and nstreams in [1, 64]");
  px_ready_ = false;  // until this run has completed
  const CublasApi &cb = cublas_api();
  GWGB_REQUIRE(cb.ok, GWGB_E_UNSUPPORTED, "libcublas could not be loaded for the reference-GPU proxy");
  const Lay &l = l_;
  const int nk = l.nk, ink = l.ink, ns = ns_, nts = nts_, half = nts_ / 2;
  const int64_t fa = l.flat_ao, fq = l.flat_aux;
  GWGB_CUDA(cudaStreamSynchronize(st_));
  check_device_flags();

  // full-BZ G in the reference's device layout [k][t][s][kslice(k)], and its tau reversal
  std::vector<int64_t> goff(nk + 1, 0);
  for (int k = 0; k < nk; ++k) goff[k + 1] = goff[k] + (int64_t)nts * ns * l.kao_sz[k];
  int64_t max_pair = 1, max_blk = 1, max_qs = 1, max_ks = 1;
  for (int p = 0; p < nk * nk; ++p) {
    max_pair = std::max<int64_t>(max_pair, (p + 1 < nk * nk ? l.kp_off[p + 1] : l.flat_V) - l.kp_off[p]);
    const int k1 = p / nk, k2 = p % nk;
    for (int b = l.kp_ptr[p]; b < l.kp_ptr[p + 1]; ++b)
      max_blk = std::max<int64_t>(max_blk, (int64_t)l.max_aux * l.aosz(k1, l.ti[3 * b + 1]) * l.aosz(k2, l.ti[3 * b + 2]));
  }
  for (int q = 0; q < nk; ++q) max_qs = std::max<int64_t>(max_qs, l.qaux_sz[q]);
  for (int k = 0; k < nk; ++k) max_ks = std::max<int64_t>(max_ks, l.kao_sz[k]);
  // cuBLAS takes 32-bit counts (AXPY / SCAL lengths, matrix sizes)
  const int64_t imax = 2147483647;
  GWGB_REQUIRE((int64_t)nts * fq <= imax && (int64_t)nts * ns * fa <= imax && max_pair <= imax &&
                   (int64_t)nts * ns * max_ks <= imax,
               GWGB_E_UNSUPPORTED, "layout too large for the 32-bit cuBLAS calls of the reference-GPU proxy");
  const int S = nstreams;
  DBuf<double2> gfull, grev, vt, vc, x1, x2, plocal, prot, slocal, pacc, sacc, rt;
  const int64_t max_rt = std::max<int64_t>((int64_t)nts * ns * l.max_ao * l.max_ao, (int64_t)nts * l.max_aux * l.max_aux);
  rt.alloc((size_t)(S * max_rt));
  gfull.alloc((size_t)goff[nk]);
  grev.alloc((size_t)goff[nk]);
  vt.alloc((size_t)(S * max_pair));
  vc.alloc((size_t)(S * max_pair));
  x1.alloc((size_t)(S * nt_batch * max_blk));
  x2.alloc((size_t)(S * nt_batch * max_blk));
  plocal.alloc((size_t)(S * nt_batch * max_qs));
  prot.alloc((size_t)(S * nts * max_qs));
  slocal.alloc((size_t)(S * nts * ns * max_ks));
  pacc.alloc((size_t)(S * nts * fq));
  sacc.alloc((size_t)(S * nts * ns * fa));
  ProxyResources res(cb);
  res.ss.assign(S, nullptr);
  for (auto &s : res.ss) GWGB_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  const std::vector<cudaStream_t> &ss = res.ss;
  GWGB_CUBLAS(cb.create(&res.h));
  cublasHandle_t h = res.h;
  cudaEvent_t ef = res.event(cudaEventDisableTiming);
  cudaEvent_t e0 = res.event(cudaEventDefault), e1 = res.event(cudaEventDefault), e2 = res.event(cudaEventDefault);
  std::vector<cudaEvent_t> es(S);
  for (auto &e : es) e = res.event(cudaEventDisableTiming);
  int64_t ngemm = 0, nother = 0;
  const cuDoubleComplex one = cz(1.0), zero = cz(0.0);
  auto on = [&](int s) { GWGB_CUBLAS(cb.set_stream(h, ss[s])); };
  auto fork = [&](cudaEvent_t t) {  // t: the phase's start (timing), then the streams start
    GWGB_CUDA(cudaEventRecord(t, st_));
    GWGB_CUDA(cudaEventRecord(ef, st_));
    for (auto &s : ss) GWGB_CUDA(cudaStreamWaitEvent(s, ef, 0));
  };
  auto join = [&]() {
    for (int s = 0; s < S; ++s) {
      GWGB_CUDA(cudaEventRecord(es[s], ss[s]));
      GWGB_CUDA(cudaStreamWaitEvent(st_, es[s], 0));
    }
  };
  // dst = op(O X O^H) over a batch: X (n x n) at src + i*sstride, O (m x n), dst (m x m) at dst + i*dstride;
  // tmp holds the batch of O X
  auto rotate = [&](double2 *dst, int64_t dstride, const double2 *src, int64_t sstride, const double2 *O, int m,
                    int n, int batch, double2 *tmp) {
    // row-major T = O X: col-major T^T = X^T O^T
    GWGB_CUBLAS(cb.zgemm_sb(h, CUBLAS_OP_N, CUBLAS_OP_N, n, m, n, &one, zc(src), n, sstride, zc(O), n, 0, &zero,
                            zc(tmp), n, (int64_t)m * n, batch));
    // row-major D = T O^H
    GWGB_CUBLAS(cb.zgemm_sb(h, CUBLAS_OP_C, CUBLAS_OP_N, m, m, n, &one, zc(O), n, 0, zc(tmp), n, (int64_t)m * n,
                            &zero, zc(dst), m, dstride, batch));
    ngemm += 2;
  };
  auto conj_inplace = [&](double2 *p, int64_t n) {
    const double m1 = -1.0;
    GWGB_CUBLAS(cb.dscal(h, (int)n, &m1, reinterpret_cast<double *>(p) + 1, 2));  // imaginary parts
    ++nother;
  };

  // ---- P0 phase (with the G set-up the reference does in copy_G_host_to_device)
  fork(e0);
  GWGB_CUDA(cudaMemsetAsync(pacc.p, 0, pacc.n * sizeof(double2), ss[0]));
  GWGB_CUDA(cudaMemsetAsync(sacc.p, 0, sacc.n * sizeof(double2), ss[0]));
  on(0);
  for (int k = 0; k < nk; ++k) {  // G(k) from the irreducible G in Gall_ ([t][s][flat_ao])
    const int ck = l.conj_index[k], ick = l.irre_index[ck], kk = l.irre_list[ick];
    const int64_t ks = l.kao_sz[k];
    double2 *dst = gfull.p + goff[k];
    const double2 *src = Gall_.p + l.kao_off_irre[ick];
    if (l.index[ck] == ck) {  // a copy of the stored slice (conjugated for k != ck)
      GWGB_CUDA(cudaMemcpy2DAsync(dst, ks * sizeof(double2), src, fa * sizeof(double2), ks * sizeof(double2),
                                  (size_t)nts * ns, cudaMemcpyDeviceToDevice, ss[0]));
      ++nother;
      if (k != ck) conj_inplace(dst, (int64_t)nts * ns * ks);
    } else {
      for (int b = l.or_ptr[ck]; b < l.or_ptr[ck + 1]; ++b) {
        const int i1 = l.or_ir[2 * b], i2 = l.or_ir[2 * b + 1];
        const int m = l.aosz(ck, i1), n = l.aosz(kk, i2);
        rotate(dst + l.aooff(ck, i1), ks, src + l.aooff(kk, i2), fa, orep_.p + l.kor_off[ck] + l.or_off[b], m, n,
               nts * ns, rt.p);
      }
      if (k != ck) conj_inplace(dst, (int64_t)nts * ns * ks);
    }
  }
  for (int k = 0; k < nk; ++k)  // G(beta - tau) as its own buffer, one copy per (k, tau)
    for (int t = 0; t < nts; ++t) {
      const int64_t sl = (int64_t)ns * l.kao_sz[k];
      GWGB_CUDA(cudaMemcpyAsync(grev.p + goff[k] + t * sl, gfull.p + goff[k] + (int64_t)(nts - 1 - t) * sl,
                                sl * sizeof(double2), cudaMemcpyDeviceToDevice, ss[0]));
      ++nother;
    }
  // the other streams start once the G set-up is done (the reference does it before the pair loop)
  GWGB_CUDA(cudaEventRecord(es[0], ss[0]));
  for (int s = 1; s < S; ++s) GWGB_CUDA(cudaStreamWaitEvent(ss[s], es[0], 0));
  const double c0 = ns == 1 ? -2.0 : -1.0;
  const cuDoubleComplex cpre = cz(c0);
  int pair = 0;
  for (int iqr = 0; iqr < ink; ++iqr) {
    const int q = l.irre_list[iqr];
    const int64_t qs = l.qaux_sz[q];
    for (int k1 = 0; k1 < nk; ++k1, ++pair) {
      const int st = pair % S;
      on(st);
      const int k2 = l.mom_cons(k1, 0, q);
      const int p = k1 * nk + k2;
      double2 *vT = vt.p + st * max_pair, *vC = vc.p + st * max_pair;
      const int64_t pbase = l.kp_off[p];
      const int64_t psz = (p + 1 < nk * nk ? l.kp_off[p + 1] : l.flat_V) - pbase;
      for (int b = l.kp_ptr[p]; b < l.kp_ptr[p + 1]; ++b) {  // V_Qpm -> V_pmQ
        const int qb = l.auxsz(q, l.ti[3 * b]), b1b2 = l.aosz(k1, l.ti[3 * b + 1]) * l.aosz(k2, l.ti[3 * b + 2]);
        GWGB_CUBLAS(cb.zgeam(h, CUBLAS_OP_T, CUBLAS_OP_N, qb, b1b2, &one, zc(V_.p + pbase + l.t_off[b]), b1b2, &zero,
                             zc(vT + l.t_off[b]), qb, zc(vT + l.t_off[b]), qb));
        ++nother;
      }
      if (psz > 0) {  // conj(V_Qpm)
        GWGB_CUDA(cudaMemcpyAsync(vC, V_.p + pbase, psz * sizeof(double2), cudaMemcpyDeviceToDevice, ss[st]));
        conj_inplace(vC, psz);
        ++nother;
      }
      double2 *pl = plocal.p + (int64_t)st * nt_batch * max_qs;
      double2 *X1 = x1.p + (int64_t)st * nt_batch * max_blk, *X2 = x2.p + (int64_t)st * nt_batch * max_blk;
      for (int t0 = 0; t0 < half; t0 += nt_batch) {
        const int nb = std::min(nt_batch, half - t0);
        for (int s = 0; s < ns; ++s) {
          GWGB_CUDA(cudaMemsetAsync(pl, 0, (size_t)nb * qs * sizeof(double2), ss[st]));
          ++nother;
          for (int b = l.kp_ptr[p]; b < l.kp_ptr[p + 1]; ++b) {
            const int iq = l.ti[3 * b], i1 = l.ti[3 * b + 1], i2 = l.ti[3 * b + 2];
            const int qb = l.auxsz(q, iq), b1 = l.aosz(k1, i1), b2 = l.aosz(k2, i2);
            const int64_t ks1 = (int64_t)ns * l.kao_sz[k1], ks2 = (int64_t)ns * l.kao_sz[k2];
            const double2 *G1 = grev.p + goff[k1] + (int64_t)t0 * ks1 + (int64_t)s * l.kao_sz[k1] + l.aooff(k1, i1);
            const double2 *G2 = gfull.p + goff[k2] + (int64_t)t0 * ks2 + (int64_t)s * l.kao_sz[k2] + l.aooff(k2, i2);
            const int64_t blk = (int64_t)qb * b1 * b2;
            // X1[t][(m,Q)] = sum_p G1[t][p] V_pmQ[p][(m,Q)]
            GWGB_CUBLAS(cb.zgemm_sb(h, CUBLAS_OP_N, CUBLAS_OP_N, b2 * qb, b1, b1, &one, zc(vT + l.t_off[b]), b2 * qb,
                                    0, zc(G1), b1, ks1, &zero, zc(X1), b2 * qb, blk, nb));
            // X2[(P,t)][m] = sum_n conj(V[P][t][n]) G2[m][n]
            GWGB_CUBLAS(cb.zgemm_sb(h, CUBLAS_OP_T, CUBLAS_OP_N, b2, qb * b1, b2, &one, zc(G2), b2, ks2,
                                    zc(vC + l.t_off[b]), b2, 0, &zero, zc(X2), b2, blk, nb));
            // P0[Q][P] += c sum_(t,m) X1[(t,m)][Q] X2[P][(t,m)]
            GWGB_CUBLAS(cb.zgemm_sb(h, CUBLAS_OP_T, CUBLAS_OP_T, qb, qb, b1 * b2, &cpre, zc(X2), b1 * b2, blk,
                                    zc(X1), qb, blk, &one, zc(pl + l.auxoff(q, iq)), qb, qs, nb));
            ngemm += 3;
          }
          GWGB_CUBLAS(cb.zaxpy(h, (int)(nb * qs), &one, zc(pl), 1,
                               zc(pacc.p + (int64_t)st * nts * fq + (int64_t)nts * l.qaux_off_irre[iqr] + t0 * qs), 1));
          ++nother;
        }
      }
    }
  }
  join();

  // ---- Sigma phase (P~ of the engine's last solve, in Pall_)
  fork(e1);
  pair = 0;
  for (int ik = 0; ik < ink; ++ik) {
    const int k1 = l.irre_list[ik];
    const int64_t ks1 = l.kao_sz[k1];
    for (int q = 0; q < nk; ++q, ++pair) {
      const int st = pair % S;
      on(st);
      const int k2 = l.mom_cons(k1, q, 0);
      const int p = k1 * nk + k2;
      const int64_t qs = l.qaux_sz[q];
      // P~(q) [t][qslice(q)] from P~(q_irr)
      double2 *Pq = prot.p + (int64_t)st * nts * max_qs;
      {
        const int cq = l.conj_index[q], q_ir = l.irre_index[q], qq = l.irre_list[q_ir];
        const double2 *src = Pall_.p + (int64_t)nts * l.qaux_off_irre[q_ir];
        if (l.index[cq] == cq) {
          GWGB_CUDA(cudaMemcpyAsync(Pq, src, (size_t)nts * qs * sizeof(double2), cudaMemcpyDeviceToDevice, ss[st]));
          ++nother;
          if (q != cq) conj_inplace(Pq, (int64_t)nts * qs);
        } else {
          for (int b = l.ar_ptr[cq]; b < l.ar_ptr[cq + 1]; ++b) {
            const int i1 = l.ar_ir[2 * b], i2 = l.ar_ir[2 * b + 1];
            const int m = l.auxsz(cq, i1), n = l.auxsz(qq, i2);
            rotate(Pq + l.auxoff(cq, i1), qs, src + l.auxoff(qq, i2), l.qaux_sz[qq],
                   auxrep_.p + l.kar_off[cq] + l.ar_off[b], m, n, nts, rt.p + (int64_t)st * max_rt);
          }
          if (q != cq) conj_inplace(Pq, (int64_t)nts * qs);
        }
      }
      double2 *vT = vt.p + st * max_pair;
      const int64_t pbase = l.kp_off[p];
      for (int b = l.kp_ptr[p]; b < l.kp_ptr[p + 1]; ++b) {  // V_Qim -> V_nPj = conj-transpose
        const int qb = l.auxsz(q, l.ti[3 * b]), b1 = l.aosz(k1, l.ti[3 * b + 1]), b2 = l.aosz(k2, l.ti[3 * b + 2]);
        GWGB_CUBLAS(cb.zgeam(h, CUBLAS_OP_C, CUBLAS_OP_N, qb * b1, b2, &one, zc(V_.p + pbase + l.t_off[b]), b2, &zero,
                             zc(vT + l.t_off[b]), qb * b1, zc(vT + l.t_off[b]), qb * b1));
        ++nother;
      }
      double2 *sl = slocal.p + (int64_t)st * nts * ns * max_ks;
      GWGB_CUDA(cudaMemsetAsync(sl, 0, (size_t)nts * ns * ks1 * sizeof(double2), ss[st]));
      ++nother;
      double2 *Y1 = x1.p + (int64_t)st * nt_batch * max_blk, *Y2 = x2.p + (int64_t)st * nt_batch * max_blk;
      const cuDoubleComplex m1 = cz(-1.0);
      for (int t0 = 0; t0 < nts; t0 += nt_batch) {
        const int nb = std::min(nt_batch, nts - t0);
        for (int s = 0; s < ns; ++s)
          for (int b = l.kp_ptr[p]; b < l.kp_ptr[p + 1]; ++b) {
            const int iq = l.ti[3 * b], i1 = l.ti[3 * b + 1], i2 = l.ti[3 * b + 2];
            const int qb = l.auxsz(q, iq), b1 = l.aosz(k1, i1), b2 = l.aosz(k2, i2);
            const int64_t ks2 = (int64_t)ns * l.kao_sz[k2];
            const double2 *G2 = gfull.p + goff[k2] + (int64_t)t0 * ks2 + (int64_t)s * l.kao_sz[k2] + l.aooff(k2, i2);
            const int64_t blk = (int64_t)qb * b1 * b2;
            // Y1[(Q,i)][n] = sum_m V[(Q,i)][m] G2[m][n]
            GWGB_CUBLAS(cb.zgemm_sb(h, CUBLAS_OP_N, CUBLAS_OP_N, b2, qb * b1, b2, &one, zc(G2), b2, ks2,
                                    zc(V_.p + pbase + l.t_off[b]), b2, 0, &zero, zc(Y1), b2, blk, nb));
            // Y2[(i,n)][P] = sum_Q Y1[Q][(i,n)] P~[Q][P]
            GWGB_CUBLAS(cb.zgemm_sb(h, CUBLAS_OP_N, CUBLAS_OP_T, qb, b1 * b2, qb, &one,
                                    zc(Pq + (int64_t)t0 * qs + l.auxoff(q, iq)), qb, qs, zc(Y1), b1 * b2, blk, &zero,
                                    zc(Y2), qb, blk, nb));
            // Sigma[i][j] -= sum_(n,P) Y2[i][(n,P)] V_nPj[(n,P)][j]
            GWGB_CUBLAS(cb.zgemm_sb(h, CUBLAS_OP_N, CUBLAS_OP_N, b1, b1, b2 * qb, &m1, zc(vT + l.t_off[b]), b1, 0,
                                    zc(Y2), b2 * qb, blk, &one,
                                    zc(sl + (int64_t)t0 * ns * ks1 + (int64_t)s * ks1 + l.aooff(k1, i1)), b1,
                                    (int64_t)ns * ks1, nb));
            ngemm += 3;
          }
      }
      GWGB_CUBLAS(cb.zaxpy(h, (int)(nts * ns * ks1), &one, zc(sl), 1,
                           zc(sacc.p + (int64_t)st * nts * ns * fa + (int64_t)nts * ns * l.kao_off_irre[ik]), 1));
      ++nother;
    }
  }
  join();
  GWGB_CUDA(cudaEventRecord(e2, st_));
  GWGB_CUDA(cudaEventSynchronize(e2));
  float ms_p0 = 0.f, ms_sig = 0.f;
  GWGB_CUDA(cudaEventElapsedTime(&ms_p0, e0, e1));
  GWGB_CUDA(cudaEventElapsedTime(&ms_sig, e1, e2));

  // sum the per-stream accumulators, /nk (outside the timed region)
  GWGB_CUBLAS(cb.set_stream(h, st_));
  for (int s = 1; s < S; ++s) {
    GWGB_CUBLAS(cb.zaxpy(h, (int)(nts * fq), &one, zc(pacc.p + (int64_t)s * nts * fq), 1, zc(pacc.p), 1));
    GWGB_CUBLAS(cb.zaxpy(h, (int)(nts * ns * fa), &one, zc(sacc.p + (int64_t)s * nts * ns * fa), 1, zc(sacc.p), 1));
  }
  const double inv = 1.0 / nk;
  GWGB_CUBLAS(cb.zdscal(h, (int)(nts * fq), &inv, zc(pacc.p), 1));
  GWGB_CUBLAS(cb.zdscal(h, (int)(nts * ns * fa), &inv, zc(sacc.p), 1));
  px_p0_.alloc((size_t)(nts * fq));
  px_sig_.alloc((size_t)(nts * ns * fa));
  GWGB_CUDA(cudaMemcpyAsync(px_p0_.p, pacc.p, px_p0_.n * sizeof(double2), cudaMemcpyDeviceToDevice, st_));
  GWGB_CUDA(cudaMemcpyAsync(px_sig_.p, sacc.p, px_sig_.n * sizeof(double2), cudaMemcpyDeviceToDevice, st_));
  GWGB_CUDA(cudaStreamSynchronize(st_));
  px_ready_ = true;
  if (out) {
    out->p0_ms = ms_p0;
    out->sigma_ms = ms_sig;
    out->gemm_calls = ngemm;
    out->other_calls = nother;
  }
}

// P0 in the host layout [q_irr][t][qslice] (t < nts/2; zeros above) and Sigma
// in [t][s][flat_ao], from the proxy's device layout [k_irr][t][s][kslice].
void Engine::refproxy_get(double *P0, double *Sg) {
  GWGB_REQUIRE(px_ready_, GWGB_E_STATE, "the reference-GPU proxy has not run");
  const Lay &l = l_;
  const int nts = nts_, ns = ns_, half = nts_ / 2;
  if (P0) {
    std::vector<double2> h(px_p0_.n);
    GWGB_CUDA(cudaMemcpy(h.data(), px_p0_.p, h.size() * sizeof(double2), cudaMemcpyDeviceToHost));
    for (int iqr = 0; iqr < l.ink; ++iqr) {
      const int64_t qs = l.qaux_sz[l.irre_list[iqr]], base = (int64_t)nts * l.qaux_off_irre[iqr];
      for (int t = half; t < nts; ++t)
        for (int64_t e = 0; e < qs; ++e) h[base + t * qs + e] = make_double2(0.0, 0.0);
    }
    std::memcpy(P0, h.data(), h.size() * sizeof(double2));
  }
  if (Sg) {
    std::vector<double2> h(px_sig_.n), o(px_sig_.n);
    GWGB_CUDA(cudaMemcpy(h.data(), px_sig_.p, h.size() * sizeof(double2), cudaMemcpyDeviceToHost));
    const int64_t fa = l.flat_ao;
    for (int ik = 0; ik < l.ink; ++ik) {
      const int64_t ks = l.kao_sz[l.irre_list[ik]], src0 = (int64_t)nts * ns * l.kao_off_irre[ik];
      for (int t = 0; t < nts; ++t)
        for (int s = 0; s < ns; ++s)
          for (int64_t e = 0; e < ks; ++e)
            o[((int64_t)t * ns + s) * fa + l.kao_off_irre[ik] + e] = h[src0 + ((int64_t)t * ns + s) * ks + e];
    }
    std::memcpy(Sg, o.data(), o.size() * sizeof(double2));
  }
}

}  // namespace gwgb
