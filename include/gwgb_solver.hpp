// gwgb_solver.hpp — header-only C++ mirror of SymmetryMBPT's solver interface
// over the C ABI of gwgb.h.
//
// gb300_gw_solver has the method names and meaning of solver_block_t
// (SymmetryMBPT/include/solver/solver_block_t.h:37-65) and of the cuGW test
// hooks (SymmetryMBPT/include/solver/cugw_solver_block.h:117-180): solve(),
// solve_P0(), solve_sigma(), compute_Pq_from_P0q(), P0_q_t_QP(),
// single_prec_run(), set_shared_Coulomb(), get_iter(), name().  As in the
// reference, G(tau) and Sigma(tau) live in caller-owned host buffers
// ([nts][ns][flat_ao] complex, the reference's G_ts_kij / Sigma_ts_kij) that
// the solver reads and writes; the P0 buffer ([ink][nts][qslice]) is owned by
// the solver.  Failures throw std::runtime_error, as the reference does.
//
// The engine adds what the reference's loop lacks: dyson(mu), iteration(mu),
// find_mu(), energy() and sc_loop().
#ifndef GWGB_SOLVER_HPP
#define GWGB_SOLVER_HPP

#include <complex>
#include <cstddef>
#include <stdexcept>
#include <string>
#include <vector>

#include "gwgb.h"

namespace gwgb {

class gb300_gw_solver {
 public:
  using dcomplex = std::complex<double>;

  // params/layout as in gwgb_create; G and Sigma: the caller's host buffers
  // (nts * ns * flat_ao each); V: the flat block Coulomb integrals (flat_V
  // elements), borrowed until set_shared_Coulomb() has uploaded them.
  gb300_gw_solver(const gwgb_params &params, const gwgb_layout &layout, dcomplex *G_ts_kij, dcomplex *Sigma_ts_kij,
                  const dcomplex *V, std::size_t nV, std::size_t flat_ao, std::size_t flat_aux)
      : G_(G_ts_kij), Sigma_(Sigma_ts_kij), V_(V), nV_(nV),
        g_size_((std::size_t)params.nts * params.ns * flat_ao), p_size_((std::size_t)params.nts * flat_aux),
        P0_(p_size_) {
    check(gwgb_create(&params, &layout, &h_));
  }
  gb300_gw_solver(const gb300_gw_solver &) = delete;
  gb300_gw_solver &operator=(const gb300_gw_solver &) = delete;
  virtual ~gb300_gw_solver() { gwgb_destroy(h_); }

  // rotations and transform matrices (the reference builds them in
  // symmetry_utils_t and transformer_t); see gwgb.h for the layouts
  void set_reps(const dcomplex *orep, std::size_t no, const dcomplex *auxrep, std::size_t na) {
    check(gwgb_set_reps(h_, d(orep), (int64_t)no, d(auxrep), (int64_t)na));
  }
  void set_transforms(const dcomplex *Tnt, const dcomplex *Ttn, const dcomplex *Tnt_BF, const dcomplex *Ttn_FB,
                      const int64_t *wsample_fermi, const double *tct_first = nullptr,
                      const double *tct_last = nullptr) {
    check(gwgb_set_transforms(h_, d(Tnt), d(Ttn), d(Tnt_BF), d(Ttn_FB), wsample_fermi, tct_first, tct_last));
  }
  void set_fock(const dcomplex *F, const dcomplex *S) { check(gwgb_set_fock(h_, d(F), d(S))); }

  // ---- solver_block_t -----------------------------------------------------
  // Sigma(tau) from the caller's G(tau): overwrites the caller's Sigma buffer.
  virtual void solve() {
    check(gwgb_set_G(h_, d(G_)));
    check(gwgb_solve(h_));
    check(gwgb_get_sigma(h_, dd(Sigma_)));
    ++iter_;
  }
  virtual void get_iter(int &iter) { iter = iter_; }
  // the split-precision path with the 1e-7 Ha bound (GWGB_PREC_OZAKI)
  virtual void single_prec_run(bool run_sp) {
    check(gwgb_set_precision(h_, run_sp ? GWGB_PREC_OZAKI : GWGB_PREC_FP64));
  }
  virtual void set_shared_Coulomb() {
    if (!V_) throw std::runtime_error("gb300_gw_solver: no Coulomb integrals were given");
    check(gwgb_upload_V(h_, d(V_), (int64_t)nV_));
  }
  virtual void allocate_solver_shared_memory() {}
  virtual std::string name() const { return "GB300 GW solver (gwgb)"; }

  // ---- cuGW test hooks ----------------------------------------------------
  virtual const std::vector<dcomplex> &P0_q_t_QP() const { return P0_; }
  virtual void solve_P0() {
    check(gwgb_set_G(h_, d(G_)));
    check(gwgb_solve_P0(h_));
    check(gwgb_get_P0(h_, dd(P0_.data())));
  }
  virtual void compute_Pq_from_P0q() {
    check(gwgb_set_P0(h_, d(P0_.data())));
    check(gwgb_solve_Pq(h_));
    check(gwgb_get_P0(h_, dd(P0_.data())));
  }
  virtual void solve_sigma() {
    check(gwgb_set_G(h_, d(G_)));
    check(gwgb_set_P0(h_, d(P0_.data())));
    check(gwgb_solve_sigma(h_));
    check(gwgb_get_sigma(h_, dd(Sigma_)));
  }

  // ---- beyond the reference ----------------------------------------------
  // G(tau) from the caller's Sigma(tau) at mu (dyson_sc_block_t::compute_G).
  void dyson(double mu) {
    check(gwgb_set_sigma(h_, d(Sigma_)));
    check(gwgb_dyson(h_, mu));
    check(gwgb_get_G(h_, dd(G_)));
  }
  // solve() then Dyson at mu on resident data; G and Sigma copied back.
  void iteration(double mu) {
    check(gwgb_set_G(h_, d(G_)));
    check(gwgb_iteration(h_, mu));
    check(gwgb_get_sigma(h_, dd(Sigma_)));
    check(gwgb_get_G(h_, dd(G_)));
    ++iter_;
  }
  // Dyson with a device-side mu search on the caller's Sigma; returns mu.
  double find_mu(const gwgb_mu_search &ms, double *n_out = nullptr) {
    double mu = 0.0;
    check(gwgb_set_sigma(h_, d(Sigma_)));
    check(gwgb_find_mu(h_, &ms, &mu, n_out));
    check(gwgb_get_G(h_, dd(G_)));
    return mu;
  }
  // niter self-consistent iterations from the caller's G and Sigma.
  std::vector<gwgb_sc_record> sc_loop(int niter, double alpha, const gwgb_mu_search &ms, bool final_fp64 = false) {
    std::vector<gwgb_sc_record> rec((std::size_t)niter);
    check(gwgb_set_G(h_, d(G_)));
    check(gwgb_set_sigma(h_, d(Sigma_)));
    check(gwgb_sc_loop(h_, niter, alpha, &ms, final_fp64 ? 1 : 0, rec.data()));
    check(gwgb_get_sigma(h_, dd(Sigma_)));
    check(gwgb_get_G(h_, dd(G_)));
    iter_ += niter;
    return rec;
  }
  void set_energy_matrix(const double *M, int n) { check(gwgb_set_energy_matrix(h_, M, n)); }
  void set_hcore(const dcomplex *H) { check(gwgb_set_hcore(h_, d(H))); }
  void energy(double *e_corr, double *e_one) { check(gwgb_energy(h_, e_corr, e_one)); }
  gwgb_stats stats() const {
    gwgb_stats s{};
    check(gwgb_get_stats(h_, &s));
    return s;
  }

 private:
  static void check(int rc) {
    if (rc != GWGB_OK) throw std::runtime_error(std::string("gwgb: ") + gwgb_last_error());
  }
  static const double *d(const dcomplex *p) { return reinterpret_cast<const double *>(p); }
  static double *dd(dcomplex *p) { return reinterpret_cast<double *>(p); }

  gwgb_handle h_ = nullptr;
  dcomplex *G_;
  dcomplex *Sigma_;
  const dcomplex *V_;
  std::size_t nV_;
  std::size_t g_size_, p_size_;
  std::vector<dcomplex> P0_;
  int iter_ = 0;
};

}  // namespace gwgb

#endif  // GWGB_SOLVER_HPP
