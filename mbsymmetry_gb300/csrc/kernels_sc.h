// Self-consistent loop kernels: device-side chemical-potential search,
// linear Sigma mixing, electron count and energies.  Not in the reference
// (sc_loop_block_t keeps mu fixed and never mixes or iterates); the
// formulas are in include/gwgb.h.
#pragma once

#include "common.h"
#include "../../include/gwgb.h"

namespace gwgb {

// One AO block of one stored k and spin, for traces over the [s][flat_ao]
// layout; w = number of mesh k mapped to the stored k.
struct TrTask {
  int64_t off;  // block offset within one tau slice [s][flat_ao]
  int32_t n;    // block size
  int32_t pad;
  double w;
};

// Device state of one mu search (bracketed Illinois regula falsi).
struct MuState {
  double target, tol;
  double mu;                // trial of the pending evaluation; the final mu after the search
  double lo, hi, flo, fhi;  // bracket and N - target at its ends
  double step;              // bracket expansion step
  double best_mu, best_f;   // best trial so far (smallest |N - target|)
  int32_t have_lo, have_hi, side, evals;
  int32_t done;             // |N - target| <= tol reached: later evaluations are skipped
  int32_t pad;
};

// Reset the search; the first trial is the previous search's best mu.
void launch_mu_begin(MuState *st, double *mu_dev, double step, cudaStream_t s);

// N at the pending trial from G(beta) (Gb [ns][flat_ao]), then the next trial
// into *mu_dev; on the last evaluation *mu_dev = best mu.
void launch_mu_update(const TrTask *tasks, int ntasks, const double2 *Gb, const double2 *S, double nscale,
                      MuState *st, double *mu_dev, int last, cudaStream_t s);

// Sigma <- alpha Sigma + (1 - alpha) Sigma_old; Sigma_old <- Sigma.
void launch_mix(double2 *sig, double2 *sig_old, int64_t n, double alpha, cudaStream_t s);

// Energies and N of the resident (Sigma, G) into rec[*counter], then ++*counter.
//   Hm = M G over the interior tau rows ([ncheb][ns][flat_ao]); Hc may be NULL.
struct EnergyArgs {
  const TrTask *tasks;
  int ntasks, ncheb, nts;
  int64_t ldt;  // per-tau stride of Sigma, G and Hm (ns * flat_ao)
  const double2 *sig, *hm, *g, *f, *hc, *s;
  const MuState *st;
  const unsigned long long *leak;  // NULL without leakage
  double ecorr_scale, eone_scale, nscale;
  int precision, with_energy;
  gwgb_sc_record *rec;
  int *counter;
};
void launch_energy_record(const EnergyArgs &a, cudaStream_t s);

}  // namespace gwgb
