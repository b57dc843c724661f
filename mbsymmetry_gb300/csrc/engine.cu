// GB300 GW engine: host orchestration behind the C ABI of include/gwgb.h.
//
// One handle = one GPU, one stream.  All tensors of a GW iteration are
// resident in HBM for the handle's lifetime: V (all stored k pairs), G(tau)
// for the irreducible k plus the rotated copies of the other k, P0/P~(tau),
// Sigma(tau), the frequency-domain work buffers and the work lists of the
// kernels.  An iteration is a fixed sequence of kernel launches over static
// work lists, so it is captured once as a CUDA graph and replayed.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstddef>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <numeric>
#include <string>
#include <vector>

#include "common.h"
#include "kernels.h"
#include "kernels_tc.h"
#include "kernels_sc.h"
#include "kernels_oz.h"

namespace gwgb {

static thread_local std::string g_last_error = "";

void set_last_error(const std::string &msg) { g_last_error = msg; }

// ---------------------------------------------------------------------------
// Host copy of the layout with every derived offset (the arrays of
// symmetry_utils_t, SymmetryMBPT/src/common/symmetry_utils.cpp:96-307).
// ---------------------------------------------------------------------------
struct Lay {
  int nk = 0, ink = 0;
  std::vector<int> irre_list, index, irre_index, conj_index, q_ind, q_ind2;
  std::vector<int> ao_ptr, ao_sz, aux_ptr, aux_sz;
  std::vector<int64_t> ao_off, aux_off;
  std::vector<int64_t> kao_off, kao_sz, qaux_off, qaux_sz;    // full BZ
  std::vector<int64_t> kao_off_irre, qaux_off_irre;           // iBZ
  int64_t flat_ao = 0, flat_aux = 0, flat_ao_full = 0, flat_aux_full = 0;
  std::vector<int> kp_ptr, ti;
  std::vector<int64_t> t_off, kp_off;
  int64_t flat_V = 0;
  std::vector<int> or_ptr, or_ir, ar_ptr, ar_ir;
  std::vector<int64_t> or_off, kor_off, ar_off, kar_off;
  int64_t flat_orep = 0, flat_auxrep = 0;
  int max_ao = 0, max_aux = 0;

  int mom_cons(int i, int j, int k) const { return q_ind[k * nk + q_ind2[i * nk + j]]; }
  int aosz(int k, int b) const { return ao_sz[ao_ptr[k] + b]; }
  int auxsz(int k, int b) const { return aux_sz[aux_ptr[k] + b]; }
  int64_t aooff(int k, int b) const { return ao_off[ao_ptr[k] + b]; }
  int64_t auxoff(int k, int b) const { return aux_off[aux_ptr[k] + b]; }
  int nao_blocks(int k) const { return ao_ptr[k + 1] - ao_ptr[k]; }
  int naux_blocks(int k) const { return aux_ptr[k + 1] - aux_ptr[k]; }
};

template <typename T>
static std::vector<T> copy_vec(const int32_t *p, size_t n, const char *what) {
  GWGB_REQUIRE(p != nullptr || n == 0, GWGB_E_INVALID, std::string("layout field ") + what + " is NULL");
  std::vector<T> v(n);
  for (size_t i = 0; i < n; ++i) v[i] = (T)p[i];
  return v;
}

static Lay derive_layout(const gwgb_layout &L) {
  Lay l;
  const int nk = L.nk, ink = L.ink;
  GWGB_REQUIRE(nk > 0 && ink > 0 && ink <= nk, GWGB_E_INVALID, "nk/ink out of range");
  l.nk = nk; l.ink = ink;
  l.irre_list = copy_vec<int>(L.irre_list, ink, "irre_list");
  l.index = copy_vec<int>(L.index, nk, "index");
  l.irre_index = copy_vec<int>(L.irre_index, nk, "irre_index");
  l.conj_index = copy_vec<int>(L.conj_index, nk, "conj_index");
  l.q_ind = copy_vec<int>(L.q_ind, (size_t)nk * nk, "q_ind");
  l.q_ind2 = copy_vec<int>(L.q_ind2, (size_t)nk * nk, "q_ind2");
  for (int v : l.irre_list) GWGB_REQUIRE(v >= 0 && v < nk, GWGB_E_INVALID, "irre_list entry out of range");
  for (int v : l.index) GWGB_REQUIRE(v >= 0 && v < nk, GWGB_E_INVALID, "index entry out of range");
  for (int v : l.irre_index) GWGB_REQUIRE(v >= 0 && v < ink, GWGB_E_INVALID, "irre_index entry out of range");
  for (int v : l.conj_index) GWGB_REQUIRE(v >= 0 && v < nk, GWGB_E_INVALID, "conj_index entry out of range");
  for (int v : l.q_ind) GWGB_REQUIRE(v >= 0 && v < nk, GWGB_E_INVALID, "q_ind entry out of range");
  for (int v : l.q_ind2) GWGB_REQUIRE(v >= 0 && v < nk, GWGB_E_INVALID, "q_ind2 entry out of range");
  l.ao_ptr = copy_vec<int>(L.ao_block_ptr, nk + 1, "ao_block_ptr");
  l.aux_ptr = copy_vec<int>(L.aux_block_ptr, nk + 1, "aux_block_ptr");
  GWGB_REQUIRE(l.ao_ptr[0] == 0 && l.aux_ptr[0] == 0, GWGB_E_INVALID, "block pointer arrays must start at 0");
  for (int k = 0; k < nk; ++k)
    GWGB_REQUIRE(l.ao_ptr[k + 1] > l.ao_ptr[k] && l.aux_ptr[k + 1] > l.aux_ptr[k], GWGB_E_INVALID,
                 "every k point needs at least one AO and one aux block");
  l.ao_sz = copy_vec<int>(L.ao_sizes, l.ao_ptr[nk], "ao_sizes");
  l.aux_sz = copy_vec<int>(L.aux_sizes, l.aux_ptr[nk], "aux_sizes");
  for (int v : l.ao_sz) GWGB_REQUIRE(v > 0 && v <= MAX_BLOCK, GWGB_E_UNSUPPORTED, "AO block size outside 1..64");
  for (int v : l.aux_sz) GWGB_REQUIRE(v > 0 && v <= MAX_BLOCK, GWGB_E_UNSUPPORTED, "aux block size outside 1..64");
  l.max_ao = *std::max_element(l.ao_sz.begin(), l.ao_sz.end());
  l.max_aux = *std::max_element(l.aux_sz.begin(), l.aux_sz.end());
  l.ao_off.resize(l.ao_sz.size());
  l.aux_off.resize(l.aux_sz.size());
  l.kao_off.resize(nk); l.kao_sz.resize(nk); l.qaux_off.resize(nk); l.qaux_sz.resize(nk);
  int64_t ka = 0, qa = 0;
  int nao0 = -1, naux0 = -1;
  for (int k = 0; k < nk; ++k) {
    int64_t acc = 0;
    int nao = 0, naux = 0;
    for (int b = l.ao_ptr[k]; b < l.ao_ptr[k + 1]; ++b) { l.ao_off[b] = acc; acc += (int64_t)l.ao_sz[b] * l.ao_sz[b]; nao += l.ao_sz[b]; }
    l.kao_sz[k] = acc; l.kao_off[k] = ka; ka += acc;
    acc = 0;
    for (int b = l.aux_ptr[k]; b < l.aux_ptr[k + 1]; ++b) { l.aux_off[b] = acc; acc += (int64_t)l.aux_sz[b] * l.aux_sz[b]; naux += l.aux_sz[b]; }
    l.qaux_sz[k] = acc; l.qaux_off[k] = qa; qa += acc;
    if (k == 0) { nao0 = nao; naux0 = naux; }
    GWGB_REQUIRE(nao == nao0 && naux == naux0, GWGB_E_INVALID, "block sizes of every k must add up to the same nao/naux");
  }
  l.flat_ao_full = ka; l.flat_aux_full = qa;
  l.kao_off_irre.resize(ink); l.qaux_off_irre.resize(ink);
  ka = 0; qa = 0;
  for (int ik = 0; ik < ink; ++ik) {
    int k = l.irre_list[ik];
    l.kao_off_irre[ik] = ka; ka += l.kao_sz[k];
    l.qaux_off_irre[ik] = qa; qa += l.qaux_sz[k];
  }
  l.flat_ao = ka; l.flat_aux = qa;
  // aux blocks of q and -q must agree: V(k1, k2) is read with aux_sizes(k2-k1)
  // in P0 and aux_sizes(k1-k2) in Sigma (gw_block.cpp:23-24 vs 101-102).
  for (int q = 0; q < nk; ++q) {
    int mq = l.mom_cons(0, q, 0);
    GWGB_REQUIRE(l.naux_blocks(q) == l.naux_blocks(mq), GWGB_E_INVALID, "aux blocks of q and -q differ");
    for (int b = 0; b < l.naux_blocks(q); ++b)
      GWGB_REQUIRE(l.auxsz(q, b) == l.auxsz(mq, b), GWGB_E_INVALID, "aux blocks of q and -q differ");
  }
  // V blocks
  const int np = nk * nk;
  l.kp_ptr = copy_vec<int>(L.kpair_block_ptr, np + 1, "kpair_block_ptr");
  GWGB_REQUIRE(l.kp_ptr[0] == 0, GWGB_E_INVALID, "kpair_block_ptr must start at 0");
  for (int p = 0; p < np; ++p) GWGB_REQUIRE(l.kp_ptr[p + 1] >= l.kp_ptr[p], GWGB_E_INVALID, "kpair_block_ptr not monotone");
  l.ti = copy_vec<int>(L.tensor_irreps, 3 * (size_t)l.kp_ptr[np], "tensor_irreps");
  l.t_off.resize(l.kp_ptr[np]);
  l.kp_off.resize(np);
  int64_t va = 0;
  for (int p = 0; p < np; ++p) {
    int k1 = p / nk, k2 = p % nk;
    int q = l.mom_cons(k2, k1, 0);
    int64_t acc = 0;
    l.kp_off[p] = va;
    for (int b = l.kp_ptr[p]; b < l.kp_ptr[p + 1]; ++b) {
      int iq = l.ti[3 * b], i1 = l.ti[3 * b + 1], i2 = l.ti[3 * b + 2];
      GWGB_REQUIRE(iq >= 0 && iq < l.naux_blocks(q) && i1 >= 0 && i1 < l.nao_blocks(k1) && i2 >= 0 &&
                       i2 < l.nao_blocks(k2),
                   GWGB_E_INVALID, "tensor_irreps entry out of range");
      l.t_off[b] = acc;
      acc += (int64_t)l.auxsz(q, iq) * l.aosz(k1, i1) * l.aosz(k2, i2);
    }
    va += acc;
  }
  l.flat_V = va;
  // rotation blocks
  l.or_ptr = copy_vec<int>(L.orep_block_ptr, nk + 1, "orep_block_ptr");
  l.ar_ptr = copy_vec<int>(L.auxrep_block_ptr, nk + 1, "auxrep_block_ptr");
  l.or_ir = copy_vec<int>(L.orep_irreps, 2 * (size_t)l.or_ptr[nk], "orep_irreps");
  l.ar_ir = copy_vec<int>(L.auxrep_irreps, 2 * (size_t)l.ar_ptr[nk], "auxrep_irreps");
  l.or_off.resize(l.or_ptr[nk]); l.ar_off.resize(l.ar_ptr[nk]);
  l.kor_off.resize(nk); l.kar_off.resize(nk);
  int64_t oa = 0, aa = 0;
  for (int k = 0; k < nk; ++k) {
    int ck = l.conj_index[k];
    int kk = l.irre_list[l.irre_index[ck]];
    l.kor_off[k] = oa;
    for (int b = l.or_ptr[k]; b < l.or_ptr[k + 1]; ++b) {
      int i1 = l.or_ir[2 * b], i2 = l.or_ir[2 * b + 1];
      GWGB_REQUIRE(i1 >= 0 && i1 < l.nao_blocks(ck) && i2 >= 0 && i2 < l.nao_blocks(kk), GWGB_E_INVALID,
                   "orep_irreps entry out of range");
      l.or_off[b] = oa - l.kor_off[k];
      oa += (int64_t)l.aosz(ck, i1) * l.aosz(kk, i2);
    }
    l.kar_off[k] = aa;
    for (int b = l.ar_ptr[k]; b < l.ar_ptr[k + 1]; ++b) {
      int i1 = l.ar_ir[2 * b], i2 = l.ar_ir[2 * b + 1];
      GWGB_REQUIRE(i1 >= 0 && i1 < l.naux_blocks(ck) && i2 >= 0 && i2 < l.naux_blocks(kk), GWGB_E_INVALID,
                   "auxrep_irreps entry out of range");
      l.ar_off[b] = aa - l.kar_off[k];
      aa += (int64_t)l.auxsz(ck, i1) * l.auxsz(kk, i2);
    }
  }
  l.flat_orep = oa; l.flat_auxrep = aa;
  return l;
}

// ---------------------------------------------------------------------------
// device buffer helper
// ---------------------------------------------------------------------------
// Device bytes held by the buffers of every live handle in this process.
static std::atomic<int64_t> g_device_bytes{0};

template <typename T>
struct DBuf {
  T *p = nullptr;
  size_t n = 0;
  void alloc(size_t count) {
    free();
    if (count) GWGB_CUDA(cudaMalloc(&p, count * sizeof(T)));
    n = count;
    g_device_bytes += (int64_t)(n * sizeof(T));
  }
  void upload(const std::vector<T> &v, cudaStream_t st) {
    alloc(v.size());
    if (n) GWGB_CUDA(cudaMemcpyAsync(p, v.data(), n * sizeof(T), cudaMemcpyHostToDevice, st));
  }
  void free() {
    if (p) cudaFree(p);
    g_device_bytes -= (int64_t)(n * sizeof(T));
    p = nullptr;
    n = 0;
  }
};

// An output block of a contraction and the contributions it sums.
struct Owner {
  int64_t out;      // block base at tau = 0
  int32_t ostride;  // per-tau stride
  int32_t n;        // block size (qb for P0, b1 for Sigma)
  int32_t c0, c1;   // contribution range
  int32_t smem1;    // shared memory of one tau (complex elements)
  int32_t s;        // spin (Sigma)
};

// Cut [c0, c1) into consecutive slices of at most `target` cost (a slice
// holds at least one contribution; an empty range gives one empty slice).
static std::vector<std::pair<int, int>> split_slices(const std::vector<double> &cost, int c0, int c1,
                                                     double target) {
  std::vector<std::pair<int, int>> out;
  int a = c0;
  double acc = 0;
  for (int c = c0; c < c1; ++c) {
    if (c > a && acc + cost[c] > target) {
      out.push_back({a, c});
      a = c;
      acc = 0;
    }
    acc += cost[c];
  }
  out.push_back({a, c1});
  return out;
}

static double slice_cost(const std::vector<double> &cost, const std::pair<int, int> &r) {
  double f = 0;
  for (int c = r.first; c < r.second; ++c) f += cost[c];
  return f;
}

struct GRef {
  int64_t base;
  int32_t stride;
};

// Host-side bounds check of one work item: [begin, begin + len) must lie in a
// buffer of `size` elements.  Every task list is checked when it is built, so
// no kernel launch can read or write outside its buffers whatever the layout.
static void check_range(int64_t begin, int64_t len, int64_t size, const char *what) {
  if (begin < 0 || len < 0 || begin + len > size)
    throw Error(GWGB_E_INVALID, std::string("internal work list out of bounds: ") + what);
}

class Engine {
 public:
  Engine(const gwgb_params &p, const gwgb_layout &L);
  ~Engine();

  void set_precision(int prec) {
    GWGB_REQUIRE(prec == GWGB_PREC_FP64 || prec == GWGB_PREC_TF32X3 || prec == GWGB_PREC_BF16X3 ||
                     prec == GWGB_PREC_OZAKI,
                 GWGB_E_INVALID, "unknown precision");
    if (prec != prec_) drop_graphs();  // the captured graphs hold the old kernels
    prec_ = prec;
    if (prec_ == GWGB_PREC_OZAKI) {
      if (!oz_built_) {  // the largest chunks whose buffers fit: budget 1/4, 1/8, ... of the free memory
        oz_div_ = 4;
        while (!build_oz_lists()) {
          GWGB_REQUIRE(oz_div_ < 256, GWGB_E_UNSUPPORTED, "the sliced-precision buffers do not fit the device memory");
          oz_div_ *= 2;
        }
      }
      if (!ozVcat_.p) {
        {  // the sliced path's buffers must fit the free memory: say which take it otherwise
          const std::pair<const char *, int64_t> need[] = {
              {"Z1", oz_z1_elems_ * 16}, {"Zcat", oz_zcat_elems_ * 16}, {"W", oz_w_elems_ * 16},
              {"U", oz_u_elems_ * 16}, {"Vcat", oz_vcat_elems_ * 16}, {"Bcat", oz_bcat_elems_ * 16},
              {"VcatS", oz_vcats_elems_ * 16}, {"V blocks", oz_vz_elems_ * 16}, {"partials", oz_part_elems_ * 16},
              {"G, P~ copies", (int64_t)(Gall_.n + Pall_.n) * 16}};
          int64_t tot = 0;
          std::string msg;
          for (const auto &x : need) {
            tot += x.second;
            msg += std::string(" ") + x.first + " " + std::to_string(x.second >> 20) + " MB";
          }
          size_t free_b = 0, total_b = 0;
          GWGB_CUDA(cudaMemGetInfo(&free_b, &total_b));
          GWGB_REQUIRE(tot + (256ll << 20) <= (int64_t)free_b, GWGB_E_UNSUPPORTED,
                       "sliced-precision buffers need " + std::to_string(tot >> 20) + " MB (" + msg + " ), " +
                           std::to_string(free_b >> 20) + " MB free");
        }
        ozVcat_.alloc((size_t)oz_vcat_elems_);
        ozBcat_.alloc((size_t)oz_bcat_elems_);
        ozVcatS_.alloc((size_t)oz_vcats_elems_);
        ozZ1_.alloc((size_t)oz_z1_elems_);
        ozZcat_.alloc((size_t)oz_zcat_elems_);
        ozW_.alloc((size_t)oz_w_elems_);
        ozU_.alloc((size_t)oz_u_elems_);
        ozVz_.alloc((size_t)oz_vz_elems_);
        Gff_.alloc(Gall_.n);
        Pff_.alloc(Pall_.n);
        ozPart_.alloc((size_t)oz_part_elems_);
        oz_ready_ = false;
      }
      return;
    }
    if (prec_ != GWGB_PREC_FP64 && !Wbuf_.p && wbuf_elems_) {
      Wbuf_.alloc((size_t)wbuf_elems_);
      Bcat_.alloc((size_t)bcat_elems_);
    }
    if (prec_ != GWGB_PREC_FP64 && !Zbuf_.p && zbuf_elems_) {
      Zbuf_.alloc((size_t)zbuf_elems_);
      Vcat_.alloc((size_t)vcat_elems_);
      Ppart_.alloc((size_t)ppart_elems_);
      GWGB_CUDA(cudaMemsetAsync(Zbuf_.p, 0, Zbuf_.n * sizeof(float2), st_));   // K padding stays zero
      GWGB_CUDA(cudaMemsetAsync(Vcat_.p, 0, Vcat_.n * sizeof(float2), st_));
    }
  }
  void upload_V(const double *V, int64_t n);
  void set_reps(const double *orep, int64_t no, const double *auxrep, int64_t na);
  void set_transforms(const double *Tnt, const double *Ttn, const double *TntBF, const double *TtnFB,
                      const int64_t *ws, const double *tf, const double *tl);
  void set_fock(const double *F, const double *S);
  void set_G(const double *G);
  void get_G(double *G);
  void set_sigma(const double *S);
  void get_sigma(double *S);
  void set_P0(const double *P);
  void get_P0(double *P);
  void solve_P0();
  void solve_Pq();
  void solve_sigma();
  void solve_sigma_from_P();
  void solve();
  void dyson(double mu);
  void iteration(double mu);
  void set_hcore(const double *H);
  void set_energy_matrix(const double *M, int n);
  void find_mu(const gwgb_mu_search &ms, double *mu_out, double *n_out);
  void energy(double *e_corr, double *e_one);
  void sc_loop(int niter, double alpha, const gwgb_mu_search &ms, int final_fp64, gwgb_sc_record *out);
  void refproxy(int nt_batch, int nstreams, gwgb_proxy_stats *out);
  void hf_hartree(double *J);
  void refproxy_get(double *P0, double *S);
  void stats(gwgb_stats *out) const {
    *out = stats_;
    out->device_bytes = g_device_bytes.load();
  }
  void test_raise_status(int which) {
    GWGB_REQUIRE(which >= 0 && which <= 2, GWGB_E_INVALID, "status word must be 0, 1 or 2");
    const int one = 1;
    GWGB_CUDA(cudaMemcpy(bad_.p + which, &one, sizeof(int), cudaMemcpyHostToDevice));
  }
  void synchronize() { GWGB_CUDA(cudaStreamSynchronize(st_)); check_device_flags(); }
  int device() const { return dev_; }
  std::mutex mu_lock;

 private:
  // parameters
  int ns_, nts_, nw_, nw_b_, ncheb_, prec_, dev_;
  double beta_;
  Lay l_;
  cudaStream_t st_ = nullptr;
  int smem_bytes_ = 0, sw_cap_ = 0;
  int tune_uvt_kb_ = 0, tune_npk_ = 64, tune_waves_ = 8, tune_simt_ = 0;  // tile-shape settings (gwgb_params)
  bool have_V_ = false, have_T_ = false, have_F_ = false, have_reps_ = false;
  DBuf<double2> px_p0_, px_sig_;  // results of the reference-GPU proxy
  // Hartree term of HF: work lists, c over the q = 0 aux slice, J over the stored k
  DBuf<HcTask> hart_ct_;
  DBuf<HcItem> hart_ci_;
  DBuf<HjTask> hart_jt_;
  DBuf<HjItem> hart_ji_;
  DBuf<double2> hart_c_, hart_J_;
  bool px_ready_ = false;

  // device data
  DBuf<double2> V_, Gall_, Pall_, Sig_, Pw_, Ww_, F_, S_, orep_, auxrep_;
  DBuf<double2> Tnt_, Ttn_, TntBF_, TtnFB_;
  DBuf<double> tct_f_, tct_l_, mu_dev_;
  DBuf<int64_t> ws_;
  DBuf<int> bad_;
  DBuf<unsigned long long> leak_;
  DBuf<int64_t> qoff_irr_;
  DBuf<int32_t> qsz_irr_;
  // work lists
  DBuf<P0Tile> p0_tiles_;              // FP64: (block, tau range, contribution slice)
  DBuf<P0Contrib> p0_contribs_;
  DBuf<SigTile> sig_tiles_, sig_tiles1_;  // FP64 slices / tcgen05-path (owner, tau range) tiles
  DBuf<RedTask> p0_red_, sig_red_;       // FP64: ordered sums of the slices
  DBuf<double2> Part_;                   // FP64: partial sums of the slices
  DBuf<SigContrib> sig_contribs_;
  DBuf<RotTask> rotG_;
  DBuf<VrTask> vr_tasks_;  // Vt = op(O)^T V for every Sigma contribution
  DBuf<double2> Vt_;
  bool vt_ready_ = false;
  DBuf<TSlab> slab_p_fwd_, slab_p_bwd_, slab_s_fwd_, slab_g_bwd_;
  DBuf<InvTask> inv_w_, inv_d_;
  int p0_maxo_ = 8, sig_maxo_ = 8, rot_smem_ = 0;
  int fp64_smem_ = 0, nsm_ = 0;  // FP64 contraction CTA shared memory; SM count
  // tcgen05 Sigma path: W-GEMM tiles, conj(V) operand tasks, per-contribution W references
  DBuf<SwTile> sw_tiles_;
  DBuf<BcTask> bc_tasks_;
  DBuf<WRef> sig_wref_;
  DBuf<float2> Wbuf_, Bcat_;
  int64_t bcat_elems_ = 0;
  int sw_smem_ = 0, uv_smem_ = 0, uv_smem_small_ = 0;
  std::vector<SigTile> sig_tiles1_host_;
  std::vector<char> uv_blocked_host_;
  // tau chunks of the tensor-core operands (W for Sigma, Zcat for P0), each
  // buffer sized to tc_chunk_bytes_: [t0, t1) and the work items of the chunk
  // tiles [uv0, uv0 + nuv): nuvt tcgen05 U/Sigma tiles, then nuv_blocked and the rest SIMT tiles
  struct SigChunk { int t0, t1, uv0, nuvt, nuv_blocked, nuv, w0, nw, red0, nred; };
  int uvt_smem_ = 0;
  DBuf<RedTask> uv_red_;     // ordered sums of the FP32-stage slices, per chunk
  int64_t uv_part_need_ = 0;
  struct P0Chunk { int t0, t1, k0, nk, r0, nr; };
  std::vector<SigChunk> sig_chunks_;
  std::vector<P0Chunk> p0_chunks_;
  int tch_w_ = 1, tch_z_ = 1;
  int64_t tc_chunk_bytes_ = 1ll << 30;
  int chunk_len(int64_t elems_per_tau, int ntau) const {  // float2 elements per tau -> tau per chunk
    const int64_t t = tc_chunk_bytes_ / std::max<int64_t>(1, elems_per_tau * 8);
    return (int)std::max<int64_t>(1, std::min<int64_t>(ntau, t));
  }
  int64_t wbuf_elems_ = 0;
  // tcgen05 P0 path: Z tasks (into Zcat), Vcat tasks, split-K tiles, reduction tiles
  DBuf<PzTask> pz_tasks_;
  DBuf<VcTask> vc_tasks_;
  DBuf<PkTile> pk_tiles_;
  DBuf<PrTile> pr_tiles_;
  DBuf<float2> Zbuf_, Vcat_;
  DBuf<double2> Ppart_;
  int64_t zbuf_elems_ = 0, vcat_elems_ = 0, ppart_elems_ = 0;
  int pz_smem_ = 0;
  bool vcat_ready_ = false;
  // tau-independent operands derived from V and the rotations, built outside any
  // graph capture before a solve: Vt for Sigma (all precisions), and for the
  // tensor-core paths Vcat (P0, from V) and Bcat = conj(Vt) (Sigma)
  void prepare_operands() {
    require_ready(false);
    bool built = false;
    if (!vt_ready_) {
      launch_vrot(vr_tasks_.p, (int)vr_tasks_.n, V_.p, auxrep_.p, Vt_.p, st_);
      vt_ready_ = true;
      vcat_ready_ = false;
      built = true;
    }
    if (prec_ == GWGB_PREC_OZAKI && !oz_ready_) {
      // tau-independent operands of contractions that run in one chunk: built once per upload
      for (const OzLaunch &x : oz_static_)
        launch_oz_perm(oz_perm_.p + x.t0, (int)x.n, static_cast<const double2 *>(oz_ptr(x.a)),
                       static_cast<float4 *>(const_cast<void *>(oz_ptr(x.c))), st_);
      oz_ready_ = true;
      built = true;
    }
    if (tc_split() && !vcat_ready_) {
      launch_vcat(vc_tasks_.p, (int)vc_tasks_.n, V_.p, Vcat_.p, st_);
      launch_bcat(bc_tasks_.p, (int)bc_tasks_.n, Vt_.p, Bcat_.p, st_);
      vcat_ready_ = true;
      built = true;
    }
    if (built) GWGB_CUDA(cudaStreamSynchronize(st_));
  }
  bool tc_split() const { return prec_ == GWGB_PREC_TF32X3 || prec_ == GWGB_PREC_BF16X3; }
  // Sliced (Ozaki) path: descriptors and tasks of the six GEMM stages per tau
  // chunk, the float-float operand buffers and the copies that build the
  // tau-independent ones from V / Vt.
  // OZB_G, OZB_P: float-float copies of G and P~ (per iteration); OZB_V, OZB_VT: the
  // FP64 V and pre-rotated V (sources of the operand builds); OZB_VZ: a chunk's V blocks
  enum OzBufId { OZB_G, OZB_P, OZB_V, OZB_VT, OZB_VZ, OZB_VCAT, OZB_BCAT, OZB_VCATS, OZB_Z1, OZB_ZCAT, OZB_W, OZB_U,
                 OZB_P0, OZB_SIG };
  // one stage launch: tasks [t0, t0 + n); with nr > 0 the stage writes FP64 K-slice partials to
  // ozPart_ and the ordered sums oz_red_[r0, r0 + nr) (times scale) go to buffer c afterwards
  // simt: the CUDA-core float-float kernel; part: C is ozPart_ (K-slice partials)
  struct OzLaunch {
    int64_t t0, n;
    int a, b, c;
    bool simt = false, part = false;
    bool perm = false;        // an operand build: oz_perm_[t0, t0 + n) from buffer a into buffer c
    int64_t r0 = 0, nr = 0;
    double scale = 1.0;
    int stage = 0;            // gwgb_launch_stat.stage
    double flops = 0, ops = 0, red_bytes = 0;
    int red_ny = 1;           // CTAs per reduced block
  };
  // per-launch profile (gwgb_set_launch_timing): records [0, n_p0) P0, then Sigma
  bool lt_on_ = false, lt_ran_p0_ = false, lt_ran_sig_ = false;
  std::vector<cudaEvent_t> lt_ev_;
  std::vector<gwgb_launch_stat> lt_info_;
  int lt_n_p0_ = 0;
  void rec_ev(cudaEvent_t e) {
    if (capturing_)
      GWGB_CUDA(cudaEventRecordWithFlags(e, st_, cudaEventRecordExternal));
    else
      GWGB_CUDA(cudaEventRecord(e, st_));
  }
  void lt_build() {  // one entry per GEMM launch and per reduction, in launch order
    lt_info_.clear();
    for (int l = 0; l < 2; ++l) {
      for (const OzLaunch &x : l ? oz_sig_ : oz_p0_) {
        gwgb_launch_stat g{};
        g.stage = x.stage;
        g.kernel = x.perm ? 3 : x.simt ? 1 : 0;
        g.tasks = (int32_t)x.n;
        g.flops = x.flops;
        g.mma_flops = x.ops;
        g.bytes = x.perm ? x.red_bytes : 0.0;
        lt_info_.push_back(g);
        if (x.nr && !x.perm) {
          gwgb_launch_stat r{};
          r.stage = x.stage;
          r.kernel = 2;
          r.tasks = (int32_t)x.nr;
          r.bytes = x.red_bytes;
          lt_info_.push_back(r);
        }
      }
      if (l == 0) lt_n_p0_ = (int)lt_info_.size();
    }
  }
  void lt_free() {
    for (cudaEvent_t e : lt_ev_) cudaEventDestroy(e);
    lt_ev_.clear();
  }

 public:
  void set_launch_timing(int on) {
    GWGB_REQUIRE(on == 0 || on == 1, GWGB_E_INVALID, "launch timing must be 0 or 1");
    if ((on != 0) == lt_on_) return;
    drop_graphs();  // the captured graph holds (or lacks) the event records
    lt_on_ = on != 0;
    lt_ran_p0_ = lt_ran_sig_ = false;
  }
  void launch_stats(gwgb_launch_stat *out, int max, int *n) {
    GWGB_REQUIRE(n && (out || max == 0) && max >= 0, GWGB_E_INVALID, "bad launch-stats arguments");
    *n = (int)lt_info_.size();
    GWGB_CUDA(cudaStreamSynchronize(st_));
    for (int i = 0; i < std::min(max, (int)lt_info_.size()); ++i) {
      gwgb_launch_stat g = lt_info_[i];
      const bool ran = lt_on_ && (i < lt_n_p0_ ? lt_ran_p0_ : lt_ran_sig_) && (int)lt_ev_.size() > 2 * i + 1;
      g.ran = ran ? 1 : 0;
      g.ms = 0;
      if (ran) {
        float ms = 0;
        GWGB_CUDA(cudaEventElapsedTime(&ms, lt_ev_[2 * i], lt_ev_[2 * i + 1]));
        g.ms = ms;
      }
      out[i] = g;
    }
  }

 private:
  int oz_simt_n_ = 8;  // block GEMMs with at most this many output columns run on the CUDA cores
  bool oz_built_ = false, oz_ready_ = false;
  DBuf<OzDesc> oz_descs_;
  DBuf<OzTask> oz_tasks_;
  DBuf<int64_t> oz_rowtab_;
  DBuf<RedTask> oz_red_;
  DBuf<double2> ozPart_;
  int64_t oz_part_elems_ = 1;
  DBuf<float4> Gff_, Pff_, ozVz_, ozVcat_, ozBcat_, ozVcatS_, ozZ1_, ozZcat_, ozW_, ozU_;
  int64_t oz_vz_elems_ = 1;
  // operand builds (copies of V / Vt blocks into chunk-local Vcat, Bcat, VcatS):
  // in the launch lists per chunk, or in oz_static_ when a contraction has one chunk
  DBuf<OzPerm> oz_perm_;
  std::vector<OzLaunch> oz_static_;
  int64_t oz_vcat_elems_ = 0, oz_bcat_elems_ = 0, oz_vcats_elems_ = 0, oz_z1_elems_ = 0, oz_zcat_elems_ = 0,
          oz_w_elems_ = 0, oz_u_elems_ = 0;
  std::vector<OzLaunch> oz_p0_, oz_sig_;
  std::vector<P0Contrib> pc_host_;
  std::vector<SigContrib> sc_host_;
  std::vector<Owner> sig_own_host_;
  // Builds the lists with a chunk budget of 1/oz_div_ of the free memory; false
  // (nothing uploaded) when the buffers would take more than 85% of it.
  bool build_oz_lists();
  int oz_div_ = 4;
  bool tc_chunk_env_ = false;  // GWGB_TC_CHUNK_MB given: it caps the sliced path's chunks too
  const void *oz_ptr(int id) const {
    switch (id) {
      case OZB_G: return Gff_.p;
      case OZB_P: return Pff_.p;
      case OZB_V: return V_.p;
      case OZB_VT: return Vt_.p;
      case OZB_VZ: return ozVz_.p;
      case OZB_VCAT: return ozVcat_.p;
      case OZB_BCAT: return ozBcat_.p;
      case OZB_VCATS: return ozVcatS_.p;
      case OZB_Z1: return ozZ1_.p;
      case OZB_ZCAT: return ozZcat_.p;
      case OZB_W: return ozW_.p;
      case OZB_U: return ozU_.p;
      case OZB_P0: return Pall_.p;
      default: return Sig_.p;
    }
  }
  // rec: first profile record of this list (P0: 0, Sigma: lt_n_p0_)
  void oz_run(const std::vector<OzLaunch> &ls, int rec) {
    if (lt_on_ && lt_ev_.size() < 2 * lt_info_.size()) {
      const size_t n0 = lt_ev_.size();
      lt_ev_.resize(2 * lt_info_.size());
      for (size_t i = n0; i < lt_ev_.size(); ++i) GWGB_CUDA(cudaEventCreate(&lt_ev_[i]));
    }
    for (const OzLaunch &x : ls) {
      void *c = x.part ? static_cast<void *>(ozPart_.p) : const_cast<void *>(oz_ptr(x.c));
      const void *a = oz_ptr(x.a), *b = oz_ptr(x.b);
      const float4 *af = static_cast<const float4 *>(a), *bf = static_cast<const float4 *>(b);
      if (lt_on_) rec_ev(lt_ev_[2 * rec]);
      if (x.perm)
        launch_oz_perm(oz_perm_.p + x.t0, (int)x.n, static_cast<const double2 *>(a), static_cast<float4 *>(c), st_);
      else if (x.simt)
        launch_oz_simt(oz_descs_.p, oz_tasks_.p + x.t0, (int)x.n, af, bf, c, oz_rowtab_.p, st_);
      else
        launch_oz_gemm(oz_descs_.p, oz_tasks_.p + x.t0, (int)x.n, af, bf, c, oz_rowtab_.p, nsm_, bad_.p + 2, st_);
      if (lt_on_) rec_ev(lt_ev_[2 * rec + 1]);
      ++rec;
      if (x.nr) {
        if (lt_on_) rec_ev(lt_ev_[2 * rec]);
        launch_reduce_slices(oz_red_.p + x.r0, (int)x.nr, ozPart_.p,
                             static_cast<double2 *>(const_cast<void *>(oz_ptr(x.c))), nts_, x.scale, 0, st_,
                             x.red_ny);
        if (lt_on_) rec_ev(lt_ev_[2 * rec + 1]);
        ++rec;
      }
    }
  }
  struct P0Group { int64_t pout; int32_t pstride, qb, c0, c1; };
  std::vector<P0Group> p0_groups_;                            // host: P0 output blocks
  std::vector<int> sig_b1_;                                  // host: b1 of every Sigma contribution
  // host: (P~ block of the irreducible q', conj) -> Sigma contributions reading it
  std::map<std::pair<int64_t, int>, std::vector<int>> sig_groups_;
  int max_cols_p_ = 0, max_cols_g_ = 0;
  int64_t g_rot_off_ = 0;  // start of the rotated G copies
  double p0_flops_ = 0, sig_flops_ = 0;
  bool has_tct_ = false;
  // self-consistent loop: mu search state, G(i w) scratch of the search, G(beta),
  // previous Sigma, core H, Galitskii-Migdal weights and M G, records
  DBuf<double2> Wg_, Gb_, Sold_, Hc_, Me_, Hm_;
  DBuf<MuState> mus_;
  DBuf<gwgb_sc_record> recs_;
  DBuf<int> counter_;
  DBuf<TrTask> tr_tasks_;
  DBuf<TSlab> slab_e_;
  bool have_H_ = false, have_M_ = false;
  cudaGraphExec_t sc_exec_ = nullptr;
  double sc_alpha_ = 0.0;
  gwgb_mu_search sc_ms_{};
  cudaEvent_t sc_ev_[2] = {nullptr, nullptr};
  void drop_graphs() {
    if (graph_exec_) cudaGraphExecDestroy(graph_exec_);
    if (sc_exec_) cudaGraphExecDestroy(sc_exec_);
    graph_exec_ = sc_exec_ = nullptr;
  }
  void check_mu_search(const gwgb_mu_search &ms) const;
  void init_mu_state(const gwgb_mu_search &ms);
  void k_mu_search(const gwgb_mu_search &ms);
  void k_dyson_dev();
  void k_energy_record(bool with_energy);
  void k_sc_iteration(double alpha, const gwgb_mu_search &ms);
  template <typename F> void capture(cudaGraphExec_t *exec, F &&body);
  gwgb_sc_record read_record(int i);
  // graph
  cudaGraphExec_t graph_exec_ = nullptr;
  cudaEvent_t ev_[16];  // 0-6 stage boundaries; 8-11 inside the W~ solve, 12-14 inside Dyson
  double *mu_host_ = nullptr;
  gwgb_stats stats_{};

  void build_work_lists();
  void require_ready(bool need_T) const {
    GWGB_REQUIRE(have_V_, GWGB_E_STATE, "V has not been uploaded");
    GWGB_REQUIRE(have_reps_, GWGB_E_STATE, "rotation matrices have not been set");
    GWGB_REQUIRE(!need_T || have_T_, GWGB_E_STATE, "transform matrices have not been set");
  }
  // stage launchers (no synchronisation)
  void k_rotate_G();
  void k_p0(int mirror);
  void k_pq(bool mirror_first);
  void k_sigma();
  void k_dyson();
  // During stream capture an external record keeps the event a timing event
  // of the graph; outside capture a plain record.
  void record(int i) {
    if (capturing_)
      GWGB_CUDA(cudaEventRecordWithFlags(ev_[i], st_, cudaEventRecordExternal));
    else
      GWGB_CUDA(cudaEventRecord(ev_[i], st_));
  }
  bool capturing_ = false;
  float elapsed(int a, int b) {
    float ms = 0;
    GWGB_CUDA(cudaEventElapsedTime(&ms, ev_[a], ev_[b]));
    return ms;
  }
  void check_device_flags();
  // with_pq / with_dy: the W~ solve / Dyson of this call ran with events 8-11 / 12-14
  void finish_stats(bool with_dyson, bool with_gw, bool with_pq = false, bool with_dy = false);
  double tr_bytes_pq_ = 0, tr_bytes_dy_ = 0, tr_flops_pq_ = 0, tr_flops_dy_ = 0, solve_flops_pq_ = 0, solve_flops_dy_ = 0;
};

Engine::Engine(const gwgb_params &p, const gwgb_layout &L) {
  GWGB_REQUIRE(p.ns == 1 || p.ns == 2, GWGB_E_INVALID, "ns must be 1 or 2");
  GWGB_REQUIRE(p.nts >= 4 && p.nts % 2 == 0, GWGB_E_INVALID, "Number of tau points should be even number");
  GWGB_REQUIRE(p.nts <= 160 && p.nw > 0 && p.nw <= 160 && p.nw_b > 0 && p.nw_b <= 160, GWGB_E_UNSUPPORTED,
               "tau/frequency grids are limited to 160 points");
  GWGB_REQUIRE(p.beta > 0.0, GWGB_E_INVALID, "beta must be positive");
  ns_ = p.ns; nts_ = p.nts; nw_ = p.nw; nw_b_ = p.nw_b; ncheb_ = p.nts - 2;
  GWGB_REQUIRE(p.uvt_smem_kb == 0 || (p.uvt_smem_kb >= 60 && p.uvt_smem_kb <= 227), GWGB_E_INVALID,
               "uvt_smem_kb must be 0 or in [60, 227]");
  GWGB_REQUIRE(p.sw_npk_max == 0 || p.sw_npk_max == 16 || p.sw_npk_max == 32 || p.sw_npk_max == 64, GWGB_E_INVALID,
               "sw_npk_max must be 0, 16, 32 or 64");
  GWGB_REQUIRE(p.uv_waves >= 0 && p.uv_waves <= 16, GWGB_E_INVALID, "uv_waves must be in [0, 16]");
  GWGB_REQUIRE(p.uv_simt == 0 || p.uv_simt == 1, GWGB_E_INVALID, "uv_simt must be 0 or 1");
  GWGB_REQUIRE(p.oz_simt_cols >= -1 && p.oz_simt_cols <= 1024, GWGB_E_INVALID, "oz_simt_cols must be in [-1, 1024]");
  oz_simt_n_ = p.oz_simt_cols == 0 ? 8 : std::max(0, p.oz_simt_cols);
  tune_uvt_kb_ = p.uvt_smem_kb;
  tune_simt_ = p.uv_simt;
  if (p.sw_npk_max) tune_npk_ = p.sw_npk_max;
  if (p.uv_waves) tune_waves_ = p.uv_waves;
  beta_ = p.beta; prec_ = GWGB_PREC_FP64; dev_ = p.device;
  l_ = derive_layout(L);
  GWGB_CUDA(cudaSetDevice(dev_));
  GWGB_CUDA(cudaStreamCreateWithFlags(&st_, cudaStreamNonBlocking));
  for (auto &e : ev_) GWGB_CUDA(cudaEventCreate(&e));
  int optin = 0;
  GWGB_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev_));
  smem_bytes_ = std::min(optin, 200 * 1024);
  sw_cap_ = optin - 2048;  // the W GEMM kernel: all of it but its static shared memory
  int per_sm = 0;
  GWGB_CUDA(cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev_));
  GWGB_CUDA(cudaDeviceGetAttribute(&nsm_, cudaDevAttrMultiProcessorCount, dev_));
  set_fp64_kernel_attributes(smem_bytes_);
  fp64_smem_ = std::min(smem_bytes_, ((per_sm / 2 - 2048) / 1024) * 1024);  // two CTAs per SM
  set_tc_kernel_attributes(smem_bytes_, sw_cap_);
  set_tc_p0_kernel_attributes(smem_bytes_);
  set_oz_kernel_attributes();
  GWGB_CUDA(cudaMallocHost(&mu_host_, sizeof(double)));
  // device memory for one tau chunk of each tensor-core operand buffer (W, Zcat):
  // an eighth of the free memory, 1 to 16 GiB, unless GWGB_TC_CHUNK_MB says otherwise
  {
    size_t free_b = 0, total_b = 0;
    GWGB_CUDA(cudaMemGetInfo(&free_b, &total_b));
    tc_chunk_bytes_ = std::max<int64_t>(1ll << 30, std::min<int64_t>(16ll << 30, (int64_t)(free_b / 8)));
  }
  if (const char *e = std::getenv("GWGB_TC_CHUNK_MB")) {
    const long long mb = std::atoll(e);
    GWGB_REQUIRE(mb >= 1, GWGB_E_INVALID, "GWGB_TC_CHUNK_MB must be a positive integer");
    tc_chunk_bytes_ = (int64_t)mb << 20;
    tc_chunk_env_ = true;
  }
  build_work_lists();
  if (p.precision != GWGB_PREC_FP64) set_precision(p.precision);
  // buffers
  const int64_t fa = l_.flat_ao, fq = l_.flat_aux;
  V_.alloc(l_.flat_V);
  Sig_.alloc((size_t)nts_ * ns_ * fa);
  Pw_.alloc((size_t)nw_b_ * fq);
  Ww_.alloc((size_t)nw_ * ns_ * fa);
  F_.alloc((size_t)ns_ * fa);
  S_.alloc((size_t)ns_ * fa);
  orep_.alloc(l_.flat_orep);
  auxrep_.alloc(l_.flat_auxrep);
  mu_dev_.alloc(1);
  bad_.alloc(4);
  leak_.alloc(2);
  Wg_.alloc((size_t)nw_ * ns_ * fa);
  Gb_.alloc((size_t)ns_ * fa);
  Sold_.alloc((size_t)nts_ * ns_ * fa);
  Hm_.alloc((size_t)ncheb_ * ns_ * fa);
  mus_.alloc(1);
  counter_.alloc(1);
  recs_.alloc(16);
  for (auto &e : sc_ev_) GWGB_CUDA(cudaEventCreate(&e));
  GWGB_CUDA(cudaMemsetAsync(Gall_.p, 0, Gall_.n * sizeof(double2), st_));
  GWGB_CUDA(cudaMemsetAsync(Pall_.p, 0, Pall_.n * sizeof(double2), st_));
  GWGB_CUDA(cudaMemsetAsync(Sig_.p, 0, Sig_.n * sizeof(double2), st_));
  GWGB_CUDA(cudaMemsetAsync(bad_.p, 0, 4 * sizeof(int), st_));
  GWGB_CUDA(cudaStreamSynchronize(st_));
}

Engine::~Engine() {
  if (st_) cudaStreamSynchronize(st_);
  drop_graphs();
  for (auto &e : ev_) if (e) cudaEventDestroy(e);
  for (auto &e : sc_ev_) if (e) cudaEventDestroy(e);
  lt_free();
  Wg_.free(); Gb_.free(); Sold_.free(); Hc_.free(); Me_.free(); Hm_.free();
  mus_.free(); recs_.free(); counter_.free(); tr_tasks_.free(); slab_e_.free();
  if (mu_host_) cudaFreeHost(mu_host_);
  DBuf<double2> *bufs[] = {&V_, &Gall_, &Pall_, &Sig_, &Pw_, &Ww_, &F_, &S_, &orep_, &auxrep_, &px_p0_, &px_sig_,
                           &Tnt_, &Ttn_, &TntBF_, &TtnFB_};
  sw_tiles_.free(); bc_tasks_.free(); sig_wref_.free(); Wbuf_.free(); Bcat_.free(); uv_red_.free();
  pz_tasks_.free(); vc_tasks_.free(); pk_tiles_.free(); pr_tiles_.free(); Zbuf_.free(); Vcat_.free(); Ppart_.free();
  oz_descs_.free(); oz_tasks_.free(); oz_perm_.free(); oz_rowtab_.free();
  for (DBuf<float4> *b : {&Gff_, &Pff_, &ozVz_, &ozVcat_, &ozBcat_, &ozVcatS_, &ozZ1_, &ozZcat_, &ozW_, &ozU_}) b->free();
  oz_red_.free(); ozPart_.free();
  for (auto *b : bufs) b->free();
  tct_f_.free(); tct_l_.free(); mu_dev_.free(); ws_.free(); bad_.free(); leak_.free();
  qoff_irr_.free(); qsz_irr_.free();
  p0_tiles_.free(); p0_contribs_.free(); sig_tiles_.free(); sig_tiles1_.free(); sig_contribs_.free();
  p0_red_.free(); sig_red_.free(); Part_.free();
  rotG_.free(); vr_tasks_.free(); Vt_.free(); slab_p_fwd_.free(); slab_p_bwd_.free(); slab_s_fwd_.free(); slab_g_bwd_.free();
  inv_w_.free(); inv_d_.free();
  if (st_) cudaStreamDestroy(st_);
}

// ---------------------------------------------------------------------------
// work lists
// ---------------------------------------------------------------------------
void Engine::build_work_lists() {
  const Lay &l = l_;
  const int nk = l.nk, ink = l.ink;
  const int64_t fa = l.flat_ao, fq = l.flat_aux;

  // --- G references: irreducible k read in place from the host-layout
  //     buffer, every other k from its rotated copy [k'][t][s][kslice].
  std::vector<GRef> gref(nk);
  std::vector<RotTask> rg;
  g_rot_off_ = (int64_t)nts_ * ns_ * fa;
  int64_t go = g_rot_off_;
  rot_smem_ = 0;
  for (int k = 0; k < nk; ++k) {
    const int ck = l.conj_index[k];
    const int ick = l.irre_index[ck];
    const int kk = l.irre_list[ick];
    if (l.index[ck] == ck && k == ck && kk == k) {
      gref[k] = {l.kao_off_irre[ick], (int32_t)fa};
      continue;
    }
    gref[k] = {go, (int32_t)l.kao_sz[k]};
    if (l.index[ck] == ck) {
      GWGB_REQUIRE(l.kao_sz[k] == l.kao_sz[kk], GWGB_E_INVALID, "k slice size differs from its representative");
      rg.push_back({go, l.kao_off_irre[ick], 0, (int32_t)l.kao_sz[k], (int32_t)fa, (int32_t)l.kao_sz[k], 0, 0,
                    (int32_t)(k != ck)});
    } else {
      std::vector<int> covered(l.nao_blocks(ck), 0);
      for (int b = l.or_ptr[ck]; b < l.or_ptr[ck + 1]; ++b) {
        int i1 = l.or_ir[2 * b], i2 = l.or_ir[2 * b + 1];
        int m = l.aosz(ck, i1), n = l.aosz(kk, i2);
        GWGB_REQUIRE(m == n, GWGB_E_INVALID, "orep block must be square");
        covered[i1]++;
        rg.push_back({go + l.aooff(ck, i1), l.kao_off_irre[ick] + l.aooff(kk, i2), l.kor_off[ck] + l.or_off[b],
                      (int32_t)l.kao_sz[k], (int32_t)fa, m, n, 1, (int32_t)(k != ck)});
        rot_smem_ = std::max(rot_smem_, (int)((2 * m * n + n * n) * sizeof(double2)));
      }
      for (int c : covered) GWGB_REQUIRE(c == 1, GWGB_E_INVALID, "orep must map every block of k exactly once");
    }
    go += (int64_t)nts_ * ns_ * l.kao_sz[k];
  }
  Gall_.alloc((size_t)go);
  GWGB_CUDA(cudaMemsetAsync(Gall_.p, 0, Gall_.n * sizeof(double2), st_));  // defined (zero) before set_G

  // --- P sources.  Sigma reads P~(q) only as V P~(q) V^H.  With P~(q) =
  //     O P~(q') O^H for the irreducible q' (conjugated for a time-reversal
  //     partner; cugw_qkpt_block.cu:288-340), that is Vt P~(q') Vt^H with
  //     Vt = op(O)^T V, so every q reads the block of its q' directly, the
  //     Sigma contributions use pre-rotated V (built once per V / rep upload)
  //     and no rotated copy of P~ exists.
  struct PSrc { int64_t base; int32_t stride; int64_t o; int32_t conj; };
  std::vector<std::vector<PSrc>> psrc(nk);
  for (int q = 0; q < nk; ++q) {
    const int cq = l.conj_index[q];
    const int q_ir = l.irre_index[q];  // cugw_qkpt_block.cu:147
    const int qq = l.irre_list[q_ir];
    const int64_t src = (int64_t)nts_ * l.qaux_off_irre[q_ir];
    const int32_t stride = (int32_t)l.qaux_sz[qq];
    psrc[q].assign(l.naux_blocks(q), PSrc{-1, 0, -1, 0});
    if (l.index[cq] == cq && q == cq && qq == q) {
      for (int iq = 0; iq < l.naux_blocks(q); ++iq) psrc[q][iq] = {src + l.auxoff(q, iq), stride, -1, 0};
    } else if (l.index[cq] == cq) {  // the same slice, conjugated for q != cq
      GWGB_REQUIRE(l.qaux_sz[q] == l.qaux_sz[qq] && l.naux_blocks(q) == l.naux_blocks(qq), GWGB_E_INVALID,
                   "q slice differs from its representative");
      for (int iq = 0; iq < l.naux_blocks(q); ++iq) {
        GWGB_REQUIRE(l.auxsz(q, iq) == l.auxsz(qq, iq), GWGB_E_INVALID, "q block differs from its representative");
        psrc[q][iq] = {src + l.auxoff(qq, iq), stride, -1, (int32_t)(q != cq)};
      }
    } else {
      std::vector<int> covered(l.naux_blocks(cq), 0);
      for (int b = l.ar_ptr[cq]; b < l.ar_ptr[cq + 1]; ++b) {
        const int i1 = l.ar_ir[2 * b], i2 = l.ar_ir[2 * b + 1];
        GWGB_REQUIRE(l.auxsz(cq, i1) == l.auxsz(qq, i2) && l.auxsz(q, i1) == l.auxsz(cq, i1), GWGB_E_INVALID,
                     "auxrep block must be square");
        covered[i1]++;
        psrc[q][i1] = {src + l.auxoff(qq, i2), stride, l.kar_off[cq] + l.ar_off[b], (int32_t)(q != cq)};
      }
      for (int c : covered) GWGB_REQUIRE(c == 1, GWGB_E_INVALID, "auxrep must map every block of q exactly once");
    }
  }
  const int64_t po = (int64_t)nts_ * fq;
  Pall_.alloc((size_t)po);
  GWGB_CUDA(cudaMemsetAsync(Pall_.p, 0, Pall_.n * sizeof(double2), st_));

  {  // Hartree term: q = 0 V blocks with equal AO blocks on both sides
    int q0 = -1;
    for (int q = 0; q < nk && q0 < 0; ++q)
      if (l.mom_cons(0, 0, q) == 0) q0 = q;
    GWGB_REQUIRE(q0 >= 0, GWGB_E_INVALID, "the k mesh has no zero-momentum point");
    std::vector<HcTask> ct;
    std::vector<HcItem> ci;
    std::vector<HjTask> jt;
    std::vector<HjItem> ji;
    for (int iq = 0; iq < l.naux_blocks(q0); ++iq) {
      const int i0 = (int)ci.size();
      for (int k = 0; k < nk; ++k) {
        const int p = k * nk + k;
        for (int b = l.kp_ptr[p]; b < l.kp_ptr[p + 1]; ++b) {
          if (l.ti[3 * b] != iq || l.ti[3 * b + 1] != l.ti[3 * b + 2]) continue;
          const int i1 = l.ti[3 * b + 1];
          ci.push_back({l.kp_off[p] + l.t_off[b], gref[k].base + l.aooff(k, i1), gref[k].stride, l.aosz(k, i1)});
        }
      }
      ct.push_back({l.auxoff(q0, iq), l.auxsz(q0, iq), i0, (int)ci.size(), 0});
    }
    for (int ik = 0; ik < ink; ++ik) {
      const int k = l.irre_list[ik], p = k * nk + k;
      for (int i1 = 0; i1 < l.nao_blocks(k); ++i1) {
        const int i0 = (int)ji.size();
        for (int b = l.kp_ptr[p]; b < l.kp_ptr[p + 1]; ++b) {
          if (l.ti[3 * b + 1] != i1 || l.ti[3 * b + 2] != i1) continue;
          const int iq = l.ti[3 * b];
          ji.push_back({l.kp_off[p] + l.t_off[b], l.auxoff(q0, iq), l.auxsz(q0, iq), 0});
        }
        jt.push_back({l.kao_off_irre[ik] + l.aooff(k, i1), l.aosz(k, i1), i0, (int)ji.size(), 0});
      }
    }
    const int64_t qs0 = l.qaux_sz[q0];
    for (const HcTask &t : ct) {
      check_range(t.cout, t.qb, qs0, "Hartree c block");
      for (int i = t.i0; i < t.i1; ++i) {
        const HcItem &x = ci[i];
        check_range(x.v, (int64_t)t.qb * x.b * x.b, l.flat_V, "Hartree V block");
        check_range(x.g, (int64_t)(ns_ - 1) * x.gstride + (int64_t)x.b * x.b, go, "Hartree rho block");
      }
    }
    for (const HjTask &t : jt) {
      check_range(t.out, (int64_t)t.b * t.b, fa, "Hartree J block");
      for (int i = t.i0; i < t.i1; ++i) {
        const HjItem &x = ji[i];
        check_range(x.v, (int64_t)x.qb * t.b * t.b, l.flat_V, "Hartree V block");
        check_range(x.c, x.qb, qs0, "Hartree c block");
      }
    }
    hart_ct_.upload(ct, st_);
    hart_ci_.upload(ci, st_);
    hart_jt_.upload(jt, st_);
    hart_ji_.upload(ji, st_);
    hart_c_.alloc((size_t)std::max<int64_t>(1, qs0));
    hart_J_.alloc((size_t)std::max<int64_t>(1, fa));
  }
  for (const RotTask &t : rg) {  // G rotations: batch = nts * ns
    const int64_t nb = (int64_t)nts_ * ns_;
    check_range(t.dst, (nb - 1) * t.dstride + (t.rotate ? (int64_t)t.m * t.m : t.m), go, "G rotation target");
    check_range(t.src, (nb - 1) * t.sstride + (t.rotate ? (int64_t)t.n * t.n : t.m), go, "G rotation source");
    if (t.rotate) check_range(t.o, (int64_t)t.m * t.n, l.flat_orep, "orep block");
  }
  rotG_.upload(rg, st_);

  // --- P0: owner = (q_irr, aux block iq); the FP64 tiles are (owner, tau
  //     range, slice of the owner's contributions), see make_fp64_tiles.
  std::vector<P0Contrib> pc;
  std::vector<double> pcost;  // flops per contribution and tau (all spins)
  std::vector<Owner> p0_own;
  p0_flops_ = 0;
  const int half = nts_ / 2;
  for (int iqr = 0; iqr < ink; ++iqr) {
    const int q = l.irre_list[iqr];
    for (int iq = 0; iq < l.naux_blocks(q); ++iq) {
      const int qb = l.auxsz(q, iq);
      const int c0 = (int)pc.size();
      int b2max = 1;
      for (int k1 = 0; k1 < nk; ++k1) {
        const int k2 = l.mom_cons(k1, 0, q);  // k2 = k1 + q (cugw_routines_block.cu:283)
        const int p = k1 * nk + k2;
        for (int b = l.kp_ptr[p]; b < l.kp_ptr[p + 1]; ++b) {
          if (l.ti[3 * b] != iq) continue;
          const int i1 = l.ti[3 * b + 1], i2 = l.ti[3 * b + 2];
          const int b1 = l.aosz(k1, i1), b2 = l.aosz(k2, i2);
          pc.push_back({l.kp_off[p] + l.t_off[b], gref[k1].base + l.aooff(k1, i1), gref[k2].base + l.aooff(k2, i2),
                        gref[k1].stride, gref[k2].stride, b1, b2});
          const double f = 8.0 * ns_ *
                           ((double)b2 * qb * b1 * b1 + (double)qb * b1 * b2 * b2 + (double)qb * qb * b1 * b2);
          pcost.push_back(f);
          p0_flops_ += f * half;
          b2max = std::max(b2max, b2);
        }
      }
      const int c1 = (int)pc.size();
      const int64_t pout = (int64_t)nts_ * l.qaux_off_irre[iqr] + l.auxoff(q, iq);
      p0_groups_.push_back({pout, (int32_t)l.qaux_sz[q], qb, c0, c1});
      p0_own.push_back({pout, (int32_t)l.qaux_sz[q], qb, c0, c1, 2 * qb * b2max, 0});
    }
  }
  for (const Owner &o : p0_own)
    for (int c = o.c0; c < o.c1; ++c) {
      const P0Contrib &cb = pc[c];
      check_range(cb.v, (int64_t)o.n * cb.b1 * cb.b2, l.flat_V, "P0 V block");
      const int64_t last = (int64_t)(nts_ - 1) * ns_ + (ns_ - 1);
      check_range(cb.ga, last * cb.sa + (int64_t)cb.b1 * cb.b1, go, "P0 G(k1) block");
      check_range(cb.gb, last * cb.sb + (int64_t)cb.b2 * cb.b2, go, "P0 G(k2) block");
    }
  p0_contribs_.upload(pc, st_);

  {  // tcgen05 P0: per aux block, Zcat[(tau,P)][K] and Vcat[Q][K] with K over (contribution, spin);
     // Zcat holds one chunk of tau at a time (tch_z_ values), sized to the chunk budget
    std::vector<PzTask> zt;
    std::vector<VcTask> vt;
    std::vector<PkTile> kt;
    std::vector<PrTile> rt;
    int zneed = 0;
    int zcap = 110 * 1024;  // two CTAs per SM when the one-row minimum of every task fits
    struct ZGroup { int qb, zld; int64_t zoff, voff; };
    std::vector<ZGroup> zg;
    int64_t zrow = 0, voff = 0;
    for (const auto &g : p0_groups_) {
      int kofs = 0;
      for (int c = g.c0; c < g.c1; ++c) kofs += ns_ * pc[c].b1 * pc[c].b2;
      const int zld = ((kofs + 15) / 16) * 16;
      zg.push_back({g.qb, zld, zrow, voff});
      zrow += (int64_t)g.qb * zld;
      voff += (int64_t)g.qb * zld;
    }
    // K slices of 8 chunks of 16 complex columns: FP32 (TMEM) accumulation stays
    // within about one contribution, FP64 across slices.  The tau chunk is sized so
    // that both Zcat and the FP64 slice partials of one chunk fit the budget.
    const int SL = 8;
    int64_t ppart_per_tau = 0;
    for (size_t gi = 0; gi < p0_groups_.size(); ++gi) {
      const int nchunks = zg[gi].zld / 16;
      ppart_per_tau += (int64_t)p0_groups_[gi].qb * p0_groups_[gi].qb * std::max(1, (nchunks + SL - 1) / SL);
    }
    tch_z_ = chunk_len(zrow + 2 * ppart_per_tau, half);
    for (size_t gi = 0; gi < p0_groups_.size(); ++gi) {
      const auto &g = p0_groups_[gi];
      const int qb = g.qb, zld = zg[gi].zld;
      const int64_t zoff = zg[gi].zoff * tch_z_;  // group block: tch_z_ rows of qb x zld
      int zcol = 0;
      for (int c = g.c0; c < g.c1; ++c) {
        const P0Contrib &cb = pc[c];
        const int b1b2 = cb.b1 * cb.b2;
        for (int s = 0; s < ns_; ++s, zcol += b1b2) {
          zt.push_back({cb.v, cb.ga, cb.gb, zoff, cb.sa, cb.sb, cb.b1, cb.b2, qb, s, zld, zcol});
          vt.push_back({cb.v, zg[gi].voff, qb, b1b2, zld, zcol});
        }
        zneed = std::max(zneed, 8 * (cb.b2 * cb.b2 + cb.b1 * cb.b1 + 2 * b1b2 * qb));
        GWGB_REQUIRE(8 * (cb.b2 * cb.b2 + cb.b1 * cb.b1 + 2 * b1b2) <= smem_bytes_, GWGB_E_UNSUPPORTED,
                     "P0 block too large for the tcgen05 path");
        if (8 * (cb.b2 * cb.b2 + cb.b1 * cb.b1 + 2 * b1b2) > zcap) zcap = smem_bytes_;
      }
      const int NP = ((2 * qb + 15) / 16) * 16;
      GWGB_REQUIRE(NP <= 128, GWGB_E_UNSUPPORTED, "aux block too large for the tcgen05 P0 kernel");
    }
    const int64_t zbuf = zrow * tch_z_;
    int64_t ppart_max = 0;
    p0_chunks_.clear();
    for (int c0 = 0; c0 < half; c0 += tch_z_) {
      const int c1 = std::min(half, c0 + tch_z_);
      const size_t k0 = kt.size(), r0 = rt.size();
      int64_t poff = 0;  // the partial sums of one chunk, summed before the next chunk
      for (size_t gi = 0; gi < p0_groups_.size(); ++gi) {
        const auto &g = p0_groups_[gi];
        const int qb = g.qb, zld = zg[gi].zld;
        const int64_t zoff = zg[gi].zoff * tch_z_;
        const int nchunks = zld / 16;
        const int nslice = std::max(1, (nchunks + SL - 1) / SL);
        const int nt = std::max(1, std::min(c1 - c0, 128 / qb));
        const int NP = ((2 * qb + 15) / 16) * 16;
        for (int t0 = c0; t0 < c1; t0 += nt) {
          const int n = std::min(nt, c1 - t0);
          const int64_t slice = (int64_t)n * qb * qb;
          for (int sl = 0; sl < nslice; ++sl) {
            const PkTile t{zoff, zg[gi].voff, poff + sl * slice, zld, qb, t0, n, sl * SL,
                           std::max(0, std::min(SL, nchunks - sl * SL)), NP, 0};
            check_range(t.z, (int64_t)(t.t0 - c0 + t.nt) * t.qb * t.zld, zbuf, "P0 tensor-core A tile");
            GWGB_REQUIRE(t.nt * t.qb <= 128 && t.np <= 128 && (t.kc0 + t.kcn) * 16 <= t.zld, GWGB_E_INVALID,
                         "internal work list out of bounds: P0 tensor-core tile shape");
            kt.push_back(t);
          }
          rt.push_back({poff, g.pout, g.pstride, qb, t0, n, nslice, 0});
          poff += nslice * slice;
        }
      }
      ppart_max = std::max(ppart_max, poff);
      std::stable_sort(kt.begin() + k0, kt.end(), [](const PkTile &a, const PkTile &b) { return a.kcn > b.kcn; });
      p0_chunks_.push_back({c0, c1, (int)k0, (int)(kt.size() - k0), (int)r0, (int)(rt.size() - r0)});
    }
    const int64_t poff = ppart_max;
    for (const PzTask &t : zt)
      check_range(t.z + t.zcol, ((int64_t)(tch_z_ - 1) * t.qb + (t.qb - 1)) * t.zld + (int64_t)t.b1 * t.b2, zbuf,
                  "Z operand rows");
    for (const VcTask &t : vt) check_range(t.vc + t.zcol, (int64_t)(t.qb - 1) * t.zld + t.b1b2, voff, "V operand rows");
    for (const PkTile &t : kt) {
      check_range(t.vc, (int64_t)t.qb * t.zld, voff, "P0 tensor-core B tile");
      check_range(t.part, (int64_t)t.nt * t.qb * t.qb, poff, "P0 tensor-core partials");
    }
    for (const PrTile &t : rt) check_range(t.part, (int64_t)t.nslice * t.nt * t.qb * t.qb, poff, "P0 partial sums");
    pz_tasks_.upload(zt, st_);
    vc_tasks_.upload(vt, st_);
    pk_tiles_.upload(kt, st_);
    pr_tiles_.upload(rt, st_);
    zbuf_elems_ = zbuf;
    vcat_elems_ = voff;
    ppart_elems_ = poff;
    pz_smem_ = std::min(zcap, std::max(16 * 1024, ((zneed + 1023) / 1024) * 1024));
  }


  // --- Sigma: owner = (k_irr, AO block i1, spin)
  std::vector<SigContrib> sc;
  std::vector<VrTask> vr;
  int64_t vt_elems = 0;
  std::vector<double> scost;  // flops per contribution and tau
  std::vector<Owner> sig_own;
  std::vector<SigTile> stl;   // (owner, tau range) tiles of the tcgen05 path
  sig_flops_ = 0;
  for (int ik = 0; ik < ink; ++ik) {
    const int k1 = l.irre_list[ik];
    for (int i1 = 0; i1 < l.nao_blocks(k1); ++i1) {
      const int b1 = l.aosz(k1, i1);
      const int c0 = (int)sc.size();
      int qbmax = 1;
      for (int q = 0; q < nk; ++q) {
        const int k2 = l.mom_cons(k1, q, 0);  // k2 = k1 - q (cugw_routines_block.cu:307)
        const int p = k1 * nk + k2;
        for (int b = l.kp_ptr[p]; b < l.kp_ptr[p + 1]; ++b) {
          if (l.ti[3 * b + 1] != i1) continue;
          const int iq = l.ti[3 * b], i2 = l.ti[3 * b + 2];
          const int qb = l.auxsz(q, iq), b2 = l.aosz(k2, i2);
          const PSrc &ps = psrc[q][iq];
          GWGB_REQUIRE(ps.base >= 0, GWGB_E_INVALID, "aux block without a source in the irreducible q");
          vr.push_back({l.kp_off[p] + l.t_off[b], vt_elems, ps.o, qb, b1 * b2, ps.conj, 0});
          sc.push_back({vt_elems, gref[k2].base + l.aooff(k2, i2), ps.base, gref[k2].stride, ps.stride, b2, qb,
                        ps.conj, 0});
          vt_elems += (int64_t)qb * b1 * b2;
          sig_b1_.push_back(b1);
          sig_groups_[std::make_pair(ps.base, (int)ps.conj)].push_back((int)sc.size() - 1);
          const double f = 8.0 * ((double)qb * b1 * b2 * b2 + (double)b1 * b2 * qb * qb + (double)b1 * b1 * b2 * qb);
          scost.push_back(f);
          sig_flops_ += f * ns_ * nts_;
          qbmax = std::max(qbmax, qb);
        }
      }
      const int c1 = (int)sc.size();
      for (int s = 0; s < ns_; ++s) {
        const int64_t out = (int64_t)s * fa + l.kao_off_irre[ik] + l.aooff(k1, i1);
        sig_own.push_back({out, (int32_t)(ns_ * fa), b1, c0, c1, 2 * qbmax * b1, s});
      }
    }
  }
  for (const VrTask &t : vr) {
    check_range(t.v, (int64_t)t.qb * t.b1b2, l.flat_V, "Sigma V block");
    check_range(t.vt, (int64_t)t.qb * t.b1b2, vt_elems, "Sigma Vt block");
    if (t.o >= 0) check_range(t.o, (int64_t)t.qb * t.qb, l.flat_auxrep, "auxrep block");
  }
  vr_tasks_.upload(vr, st_);
  Vt_.alloc((size_t)std::max<int64_t>(1, vt_elems));
  for (size_t c = 0; c < sc.size(); ++c) {
    const SigContrib &cb = sc[c];
    check_range(cb.v, (int64_t)cb.qb * sig_b1_[c] * cb.b2, vt_elems, "Sigma Vt block");
    check_range(cb.gb, ((int64_t)(nts_ - 1) * ns_ + (ns_ - 1)) * cb.sb + (int64_t)cb.b2 * cb.b2, go,
                "Sigma G(k2) block");
    check_range(cb.pq, (int64_t)(nts_ - 1) * cb.pstride + (int64_t)cb.qb * cb.qb, po, "Sigma P(q) block");
  }
  sig_contribs_.upload(sc, st_);
  {  // tcgen05 path, U/Sigma stage: (owner, tau range, contribution slice) tiles, cost-balanced to
     // about six waves per chunk of the W buffer (tch_w_ tau each); each tile writes an FP64
     // partial block, summed in order per chunk (reduce_slices_kernel)
    int64_t wrow = 0;  // W elements per tau: sum over contributions of q_b k1_b k2_b
    for (size_t c = 0; c < sc.size(); ++c) wrow += (int64_t)sc[c].qb * sig_b1_[c] * sc[c].b2;
    tch_w_ = chunk_len(wrow, nts_);
    std::vector<double> ucost(sc.size());  // FP32-stage flops per contribution and tau
    double utotal = 0;
    for (size_t c = 0; c < sc.size(); ++c) {
      ucost[c] = 8.0 * sc[c].qb * sig_b1_[c] * sc[c].b2 * (sig_b1_[c] + sc[c].b2);
      utotal += ucost[c];
    }
    // Slices depend on the per-tau cost only (tune_waves_ waves of slices per tau), never
    // on the chunk length: the order of the FP64 sums, hence every result bit, is the
    // same for any chunking.  tcgen05 tiles span up to 128 / b1 tau, SIMT tiles 4.
    const double target = utotal * ns_ / ((double)tune_waves_ * std::max(1, nsm_));
    // tcgen05 U/Sigma tiles (AO blocks up to 64; uv_simt routes every owner to the
    // SIMT kernels): tau per tile such that one aux row of the owner's largest
    // contribution fits the shared-memory budget.  Default budget 110 KB (two CTAs per
    // SM), raised (to at most 200 KB) until the tiles of owners with AO blocks of 24 and
    // more keep the full 128 / k1_b tau rows: there the 110 KB tiles hold 1-2 tau and
    // most of the 128 MMA rows idle (C4 Sigma stage 1.81 s at 110 KB, 0.99 s at
    // 200 KB).  Owners with small blocks do not raise it: their full-tau tiles (up to
    // 64 tau of G2) would take one CTA per SM for every tile (C3 iteration 0.56 s at
    // 110 KB, 0.64 s at 200 KB).  gwgb_params.uvt_smem_kb (or GWGB_UVT_SMEM_KB) sets it.
    int uvt_budget = 110 * 1024;
    for (const Owner &o : sig_own) {
      if (o.n > 64 || o.n < 24) continue;
      int b2max = 1;
      for (int c = o.c0; c < o.c1; ++c) b2max = std::max(b2max, sc[c].b2);
      const int ntf = std::max(1, std::min(nts_, 128 / o.n));
      const int64_t nd = std::max(uvt_smem(1, ntf, o.n, b2max, false), uvt_smem(1, ntf, o.n, b2max, true));
      uvt_budget = (int)std::max<int64_t>(uvt_budget, std::min<int64_t>(nd, 200 * 1024));
    }
    if (const char *e = std::getenv("GWGB_UVT_SMEM_KB")) uvt_budget = std::max(60, std::min(227, std::atoi(e))) * 1024;  // <= 4 CTAs x 128 TMEM columns
    if (tune_uvt_kb_) uvt_budget = tune_uvt_kb_ * 1024;
    uvt_budget = std::min(uvt_budget, smem_bytes_);
    std::vector<int> own_nt(sig_own.size(), 0);  // 0: SIMT tiles
    uvt_smem_ = 0;
    for (size_t oi = 0; oi < sig_own.size(); ++oi) {
      const Owner &o = sig_own[oi];
      if (o.n > 64 || tune_simt_) continue;
      int b2max = 1;
      for (int c = o.c0; c < o.c1; ++c) b2max = std::max(b2max, sc[c].b2);
      auto need = [&](int nt) {
        return (int)std::max(uvt_smem(1, nt, o.n, b2max, false), uvt_smem(1, nt, o.n, b2max, true));
      };
      int nt = std::max(1, std::min(nts_, 128 / o.n));
      while (nt > 1 && need(nt) > uvt_budget) --nt;
      if (need(nt) > smem_bytes_) continue;
      own_nt[oi] = nt;
      uvt_smem_ = std::max(uvt_smem_, std::max(uvt_budget, need(nt)));
    }
    uvt_smem_ = std::min(smem_bytes_, ((uvt_smem_ + 1023) / 1024) * 1024);
    std::vector<std::vector<std::pair<int, int>>> oslices(sig_own.size());
    for (size_t i = 0; i < sig_own.size(); ++i)
      oslices[i] = split_slices(ucost, sig_own[i].c0, sig_own[i].c1, target);
    std::vector<SigTile> all;
    std::vector<RedTask> ured;
    uv_blocked_host_.clear();
    sig_chunks_.clear();
    uv_part_need_ = 0;
    for (int c0 = 0; c0 < nts_; c0 += tch_w_) {
      const int c1 = std::min(nts_, c0 + tch_w_);
      std::vector<SigTile> stl, utl;
      int64_t part = 0;
      const int r0 = (int)ured.size();
      for (size_t oi = 0; oi < sig_own.size(); ++oi) {
        const Owner &o = sig_own[oi];
        const int bb = o.n * o.n;
        const bool tcu = own_nt[oi] > 0;
        const int nt = tcu ? std::min(own_nt[oi], c1 - c0)
                           : std::max(1, std::min(std::min(4, c1 - c0), (smem_bytes_ / 4) / (24 * bb)));
        for (int t0 = c0; t0 < c1; t0 += nt) {
          const int n = std::min(nt, c1 - t0);
          const auto &sl = oslices[oi];
          ured.push_back({part, o.out, o.ostride, bb, t0, n, (int32_t)sl.size(), 0});
          for (const auto &r : sl) {
            (tcu ? utl : stl).push_back({o.out, part, o.ostride, o.n, r.first, r.second, t0, n, o.s,
                                         (int32_t)std::min(slice_cost(ucost, r) * n / 1e3, 2e9), own_nt[oi], 0});
            part += (int64_t)n * bb;
          }
        }
      }
      uv_part_need_ = std::max(uv_part_need_, part);
      std::stable_sort(stl.begin(), stl.end(), [](const SigTile &a, const SigTile &b) { return a.cost > b.cost; });
      std::stable_sort(utl.begin(), utl.end(), [](const SigTile &a, const SigTile &b) { return a.cost > b.cost; });
      // slices whose contributions average fewer than 200 (Q, m) terms take the
      // unblocked variant (barriers dominate there); each chunk = [blocked | small]
      std::vector<SigTile> big, small;
      for (const SigTile &t : stl) {
        double k = 0;
        for (int c = t.c0; c < t.c1; ++c) k += (double)sc[c].qb * sc[c].b2;
        const bool sm = t.c1 > t.c0 && k < 200.0 * (t.c1 - t.c0);
        (sm ? small : big).push_back(t);
      }
      SigChunk ch{c0, c1, (int)all.size(), (int)utl.size(), (int)big.size(),
                  (int)(utl.size() + big.size() + small.size()), 0, 0, r0, (int)ured.size() - r0};
      for (const SigTile &t : utl) {
        GWGB_REQUIRE(t.nt * t.b1 <= 128 && t.b1 <= 64 && t.nt <= t.ntq, GWGB_E_INVALID,
                     "internal work list out of bounds: tcgen05 U/Sigma tile shape");
        all.push_back(t);
        uv_blocked_host_.push_back(2);
      }
      for (const SigTile &t : big) { all.push_back(t); uv_blocked_host_.push_back(1); }
      for (const SigTile &t : small) { all.push_back(t); uv_blocked_host_.push_back(0); }
      sig_chunks_.push_back(ch);
    }
    for (const SigTile &t : all) check_range(t.part, (int64_t)t.nt * t.b1 * t.b1, uv_part_need_, "Sigma FP32-stage partials");
    for (const RedTask &r : ured) {
      check_range(r.part, (int64_t)r.nslice * r.nt * r.elems, uv_part_need_, "Sigma FP32-stage slice sum");
      check_range(r.out, (int64_t)(r.t0 + r.nt - 1) * r.ostride + r.elems, (int64_t)nts_ * ns_ * fa,
                  "Sigma output block");
    }
    sig_tiles1_.upload(all, st_);
    sig_tiles1_host_ = all;
    uv_red_.upload(ured, st_);
  }



  // --- FP64 tiles of both contractions and their partial-sum buffer
  {
    int need = 0;  // shared memory of the largest owner at one tau
    for (const Owner &o : p0_own) need = std::max(need, 16 * o.smem1);
    for (const Owner &o : sig_own) need = std::max(need, 16 * o.smem1);
    GWGB_REQUIRE(need <= smem_bytes_, GWGB_E_UNSUPPORTED, "irrep block too large for the FP64 contraction kernels");
    if (need > fp64_smem_) fp64_smem_ = smem_bytes_;  // one CTA per SM for very large blocks
    const int cap = fp64_smem_ / (int)sizeof(double2);
    const double waves = 2.0 * 6.0 * nsm_;  // two CTAs per SM, about six waves
    int64_t part0 = 0, part1 = 0;
    std::vector<P0Tile> pt;
    std::vector<SigTile> st;
    std::vector<RedTask> pr, sr;
    p0_maxo_ = 1;
    for (const Owner &o : p0_own) {
      const int qq = o.n * o.n;
      int nt = std::max(1, std::min(half, (256 + qq - 1) / qq));
      while (nt > 1 && nt * qq > 2048) --nt;
      while (nt > 1 && o.smem1 * nt > cap) --nt;
      p0_maxo_ = std::max(p0_maxo_, (nt * qq + 255) / 256);
      for (int t0 = 0; t0 < half; t0 += nt) {
        const int n = std::min(nt, half - t0);
        const auto sl = split_slices(pcost, o.c0, o.c1, p0_flops_ / waves / n);
        pr.push_back({part0, o.out, o.ostride, qq, t0, n, (int32_t)sl.size(), 0});
        for (const auto &r : sl) {
          pt.push_back({o.out, part0, o.ostride, o.n, r.first, r.second, t0, n,
                        (int32_t)std::min(slice_cost(pcost, r) * n / 1e3, 2e9), 0});
          part0 += (int64_t)n * qq;
        }
      }
    }
    sig_maxo_ = 1;
    for (const Owner &o : sig_own) {
      const int bb = o.n * o.n;
      int nt = std::max(1, std::min(nts_, (256 + bb - 1) / bb));
      while (nt > 1 && nt * bb > 2048) --nt;
      while (nt > 1 && o.smem1 * nt > cap) --nt;
      sig_maxo_ = std::max(sig_maxo_, (nt * bb + 255) / 256);
      for (int t0 = 0; t0 < nts_; t0 += nt) {
        const int n = std::min(nt, nts_ - t0);
        const auto sl = split_slices(scost, o.c0, o.c1, sig_flops_ / waves / n);
        sr.push_back({part1, o.out, o.ostride, bb, t0, n, (int32_t)sl.size(), 0});
        for (const auto &r : sl) {
          st.push_back({o.out, part1, o.ostride, o.n, r.first, r.second, t0, n, o.s,
                        (int32_t)std::min(slice_cost(scost, r) * n / 1e3, 2e9)});
          part1 += (int64_t)n * bb;
        }
      }
    }
    GWGB_REQUIRE(p0_maxo_ <= 16 && sig_maxo_ <= 16, GWGB_E_UNSUPPORTED, "contraction output tile too large");
    std::stable_sort(pt.begin(), pt.end(), [](const P0Tile &a, const P0Tile &b) { return a.cost > b.cost; });
    std::stable_sort(st.begin(), st.end(), [](const SigTile &a, const SigTile &b) { return a.cost > b.cost; });
    p0_tiles_.upload(pt, st_);
    sig_tiles_.upload(st, st_);
    p0_red_.upload(pr, st_);
    sig_red_.upload(sr, st_);
    const int64_t npart = std::max<int64_t>(1, std::max(std::max(part0, part1), uv_part_need_));
    for (const P0Tile &t : pt) check_range(t.part, (int64_t)t.nt * t.qb * t.qb, npart, "P0 partial slice");
    for (const SigTile &t : st) check_range(t.part, (int64_t)t.nt * t.b1 * t.b1, npart, "Sigma partial slice");
    for (const RedTask &r : pr) {
      check_range(r.part, (int64_t)r.nslice * r.nt * r.elems, npart, "P0 slice sum");
      check_range(r.out, (int64_t)(nts_ - 1) * r.ostride + r.elems, po, "P0 output block");
    }
    for (const RedTask &r : sr) {
      check_range(r.part, (int64_t)r.nslice * r.nt * r.elems, npart, "Sigma slice sum");
      check_range(r.out, (int64_t)(r.t0 + r.nt - 1) * r.ostride + r.elems, (int64_t)nts_ * ns_ * fa,
                  "Sigma output block");
    }
    Part_.alloc((size_t)npart);
  }
  {  // tcgen05 Sigma: per aux block (q, iq), Bcat = conj(V) columns, Wcat = W rows (tau, Q)
    std::vector<WRef> wr(sc.size());
    std::vector<BcTask> bt;
    std::vector<SwTile> swt;
    int64_t woff = 0, boff = 0;
    int wsmem = 0, uvneed = 0;
    for (const auto &grp : sig_groups_) {
      const std::vector<int> &cs = grp.second;
      const int qb = sc[cs[0]].qb;
      const int64_t pa = sc[cs[0]].pq;
      const int pstride = sc[cs[0]].pstride;
      const int pconj = sc[cs[0]].pconj;
      int ncol = 0;
      for (int c : cs) {
        const int b1b2 = sig_b1_[c] * sc[c].b2;
        bt.push_back({sc[c].v, boff, qb, b1b2, ncol, 0});
        wr[c] = {woff + ncol, 0};  // W rows are (tau - chunk start, Q)
        ncol += b1b2;
      }
      const int ld = (ncol + 1) & ~1;  // even row stride: 16-byte W stores
      for (int c : cs) wr[c].ld = ld;
      const int KP = ((2 * qb + 7) / 8) * 8, KP16 = ((2 * qb + 15) / 16) * 16;
      // shared memory: TF32x3 2 planes x 4 B, BF16x3 3 planes x 2 B (K padded to 16)
      // (+ 18432 B of drain tiles: 4 warps x 32 rows x 36 floats)
      auto need = [&](int npk) { return 18432 + std::max(KP * (1024 + 32 * npk), KP16 * (768 + 24 * npk)); };
      int npk = tune_npk_;
      while (npk > 16 && need(npk) > sw_cap_) npk /= 2;
      GWGB_REQUIRE(need(npk) <= sw_cap_, GWGB_E_UNSUPPORTED, "aux block too large for the tcgen05 Sigma kernel");
      wsmem = std::max(wsmem, need(npk));
      const int nt = std::max(1, std::min(tch_w_, 128 / qb));
      for (const SigChunk &ch : sig_chunks_)
        for (int t0 = ch.t0; t0 < ch.t1; t0 += nt)
          swt.push_back({pa, boff, woff, pstride, qb, t0, std::min(nt, ch.t1 - t0), ncol, KP, npk, pconj, 0, ncol,
                         ld, 0});
      boff += (int64_t)ncol * qb;
      woff += (int64_t)tch_w_ * qb * ld;
    }
    int uvneed_small = 0;
    // the U/Sigma stage keeps large Q chunks (one CTA per SM measured faster than two
    // CTAs with half the chunk); the Z stage of P0 takes two CTAs per SM
    int uv_cap = smem_bytes_;
    for (size_t n = 0; n < sig_tiles1_host_.size(); ++n) {
      const SigTile &t = sig_tiles1_host_[n];
      if (uv_blocked_host_[n] == 2) continue;  // tcgen05 U/Sigma tile (sized above)
      const bool blocked = uv_blocked_host_[n] == 1;
      int b2max = 1, qbmax = 1;
      for (int c = t.c0; c < t.c1; ++c) { b2max = std::max(b2max, sc[c].b2); qbmax = std::max(qbmax, sc[c].qb); }
      // acc64, acc32, red (blocked variant only), G2
      const int fixed = 24 * t.nt * t.b1 * t.b1 + (blocked ? 256 * 16 * 8 : 0) + 8 * b2max * b2max;
      int &need = blocked ? uvneed : uvneed_small;
      need = std::max(need, fixed + 24 * t.b1 * b2max * qbmax);
      GWGB_REQUIRE(fixed + 24 * t.b1 * b2max <= smem_bytes_, GWGB_E_UNSUPPORTED,
                   "Sigma block too large for the tcgen05 path");
      if (fixed + 24 * t.b1 * b2max > uv_cap) uv_cap = smem_bytes_;
    }
    uv_smem_small_ = std::min(uv_cap, std::max(16 * 1024, ((uvneed_small + 1023) / 1024) * 1024));
    // Columns split into ranges of whole packs so that each chunk has about four
    // waves of CTAs (a CTA computes whole W entries, so the split changes no bit)
    {
      std::vector<int64_t> packs_in_chunk(sig_chunks_.size(), 0);
      for (const SwTile &t : swt) packs_in_chunk[t.t0 / tch_w_] += (t.ncol + t.npk - 1) / t.npk;
      std::vector<SwTile> split;
      for (const SwTile &t : swt) {
        const int64_t per = std::max<int64_t>(1, (packs_in_chunk[t.t0 / tch_w_] + 4 * nsm_ - 1) / (4 * std::max(1, nsm_)));
        const int64_t range = per * t.npk;
        for (int64_t c0 = 0; c0 < t.ncol; c0 += range) {
          SwTile u = t;
          u.c0 = (int32_t)c0;
          u.c1 = (int32_t)std::min<int64_t>(t.ncol, c0 + range);
          split.push_back(u);
        }
      }
      swt.swap(split);
    }
    // tiles grouped by W chunk, widest first within a chunk
    std::stable_sort(swt.begin(), swt.end(), [&](const SwTile &a, const SwTile &b) {
      const int ca = a.t0 / tch_w_, cb = b.t0 / tch_w_;
      return ca != cb ? ca < cb : (a.c1 - a.c0) > (b.c1 - b.c0);
    });
    for (SigChunk &ch : sig_chunks_) {
      ch.w0 = (int)(std::lower_bound(swt.begin(), swt.end(), ch.t0,
                                     [&](const SwTile &t, int v) { return t.t0 / tch_w_ < v / tch_w_; }) -
                    swt.begin());
      ch.nw = (int)(std::upper_bound(swt.begin(), swt.end(), ch.t0,
                                     [&](int v, const SwTile &t) { return v / tch_w_ < t.t0 / tch_w_; }) -
                    swt.begin()) - ch.w0;
    }
    for (const SwTile &t : swt) {
      const int t0c = (t.t0 / tch_w_) * tch_w_;  // chunk start
      check_range(t.wcat, (int64_t)(t.t0 - t0c + t.nt) * t.qb * t.ld, woff, "W rows");
      GWGB_REQUIRE(t.ld >= t.ncol && (t.ld & 1) == 0 && (t.wcat & 1) == 0 && (t.c0 & 1) == 0, GWGB_E_INVALID,
                   "internal work list out of bounds: W row alignment");
      GWGB_REQUIRE(0 <= t.c0 && t.c0 < t.c1 && t.c1 <= t.ncol, GWGB_E_INVALID,
                   "internal work list out of bounds: W column range");
      check_range(t.bcat, (int64_t)t.ncol * t.qb, boff, "conj(V) operand");
      GWGB_REQUIRE(t.nt * t.qb <= 128 && 2 * t.npk <= 128, GWGB_E_INVALID,
                   "internal work list out of bounds: Sigma tensor-core tile shape");
    }
    for (const BcTask &t : bt) {
      check_range(t.v, (int64_t)t.qb * t.b1b2, vt_elems, "conj(Vt) source");
      check_range(t.bcat + (int64_t)t.col0 * t.qb, (int64_t)t.b1b2 * t.qb, boff, "conj(V) target");
    }
    sw_tiles_.upload(swt, st_);
    bc_tasks_.upload(bt, st_);
    sig_wref_.upload(wr, st_);
    sw_smem_ = std::max(16 * 1024, wsmem);
    uv_smem_ = std::min(uv_cap, std::max(16 * 1024, ((uvneed + 1023) / 1024) * 1024));
    wbuf_elems_ = woff;
    bcat_elems_ = boff;
  }

  // --- transforms and block inverses
  std::vector<TSlab> pf, pb, sf, gb;
  std::vector<InvTask> iw, id;
  std::vector<int64_t> qo(ink);
  std::vector<int32_t> qs(ink);
  max_cols_p_ = max_cols_g_ = 0;
  for (int iqr = 0; iqr < ink; ++iqr) {
    const int q = l.irre_list[iqr];
    const int64_t off = l.qaux_off_irre[iqr];
    const int32_t sz = (int32_t)l.qaux_sz[q];
    qo[iqr] = off;
    qs[iqr] = sz;
    pf.push_back({(int64_t)nts_ * off, (int64_t)nw_b_ * off, sz, sz, sz, 0});
    pb.push_back({(int64_t)nw_b_ * off, (int64_t)nts_ * off, sz, sz, sz, 0});
    max_cols_p_ = std::max(max_cols_p_, (int)sz);
    for (int n = 0; n < nw_b_; ++n)
      for (int b = 0; b < l.naux_blocks(q); ++b)
        iw.push_back({(int64_t)nw_b_ * off + (int64_t)n * sz + l.auxoff(q, b), 0, 0, l.auxsz(q, b), -1});
  }
  for (int s = 0; s < ns_; ++s)
    for (int ik = 0; ik < ink; ++ik) {
      const int k = l.irre_list[ik];
      const int64_t koff = l.kao_off_irre[ik];
      const int32_t ksz = (int32_t)l.kao_sz[k];
      const int64_t wbase = (int64_t)nw_ * (s * fa + koff);
      sf.push_back({s * fa + koff, wbase, (int32_t)(ns_ * fa), ksz, ksz, 0});
      gb.push_back({wbase, s * fa + koff, ksz, (int32_t)(ns_ * fa), ksz, 0});
      max_cols_g_ = std::max(max_cols_g_, (int)ksz);
      for (int w = 0; w < nw_; ++w)
        for (int b = 0; b < l.nao_blocks(k); ++b)
          id.push_back({wbase + (int64_t)w * ksz + l.aooff(k, b), s * fa + koff + l.aooff(k, b),
                        s * fa + koff + l.aooff(k, b), l.aosz(k, b), w});
    }
  slab_p_fwd_.upload(pf, st_);
  slab_p_bwd_.upload(pb, st_);
  slab_s_fwd_.upload(sf, st_);
  slab_g_bwd_.upload(gb, st_);
  {  // traces over the stored k (weight = mesh k mapped to each) and the M G slabs
    std::vector<double> wk(ink, 0.0);
    for (int k = 0; k < nk; ++k) wk[l.irre_index[k]] += 1.0;
    std::vector<TrTask> tt;
    std::vector<TSlab> se;
    for (int s = 0; s < ns_; ++s)
      for (int ik = 0; ik < ink; ++ik) {
        const int k = l.irre_list[ik];
        const int64_t koff = s * fa + l.kao_off_irre[ik];
        se.push_back({koff, koff, (int32_t)(ns_ * fa), (int32_t)(ns_ * fa), (int32_t)l.kao_sz[k], 0});
        for (int b = 0; b < l.nao_blocks(k); ++b) tt.push_back({koff + l.aooff(k, b), l.aosz(k, b), 0, wk[ik]});
      }
    tr_tasks_.upload(tt, st_);
    slab_e_.upload(se, st_);
  }
  {
    const int64_t gsz = (int64_t)nts_ * ns_ * fa, wsz = (int64_t)nw_ * ns_ * fa, pwsz = (int64_t)nw_b_ * fq;
    auto slabs = [&](const std::vector<TSlab> &v, int nin, int row0, int64_t xs, int nout, int64_t ys, const char *w) {
      for (const TSlab &t : v) {
        check_range(t.x + (int64_t)row0 * t.ldx, (int64_t)(nin - 1) * t.ldx + t.ncols, xs, w);
        check_range(t.y, (int64_t)(nout - 1) * t.ldy + t.ncols, ys, w);
      }
    };
    slabs(pf, ncheb_, 1, po, nw_b_, pwsz, "P tau->Omega slab");
    slabs(pb, nw_b_, 0, pwsz, nts_, po, "P Omega->tau slab");
    slabs(sf, ncheb_, 1, gsz, nw_, wsz, "Sigma tau->omega slab");
    slabs(gb, nw_, 0, wsz, nts_, gsz, "G omega->tau slab");
    for (const InvTask &t : iw) check_range(t.a, (int64_t)t.n * t.n, pwsz, "W~ block");
    for (const InvTask &t : id) {
      check_range(t.a, (int64_t)t.n * t.n, wsz, "Dyson block");
      check_range(t.s, (int64_t)t.n * t.n, (int64_t)ns_ * fa, "S/F block");
    }
  }
  inv_w_.upload(iw, st_);
  inv_d_.upload(id, st_);
  {  // algorithmic work of the transforms (16 (n_in + n_out) B per column + T once per launch) and
     // of the block solves (W~: inverse + product, 16 n^3 flop; Dyson: inverse, 8 n^3)
    auto tb = [](const std::vector<TSlab> &v, int nin, int nout) {
      double b = 16.0 * nin * nout;
      for (const TSlab &t : v) b += 16.0 * (nin + nout) * t.ncols;
      return b;
    };
    tr_bytes_pq_ = tb(pf, ncheb_, nw_b_) + tb(pb, nw_b_, nts_);
    tr_bytes_dy_ = tb(sf, ncheb_, nw_) + tb(gb, nw_, nts_);
    auto tf = [](const std::vector<TSlab> &v, int nin, int nout) {  // 8 n_in n_out flop per complex column
      double f = 0;
      for (const TSlab &t : v) f += 8.0 * nin * nout * t.ncols;
      return f;
    };
    tr_flops_pq_ = tf(pf, ncheb_, nw_b_) + tf(pb, nw_b_, nts_);
    tr_flops_dy_ = tf(sf, ncheb_, nw_) + tf(gb, nw_, nts_);
    solve_flops_pq_ = solve_flops_dy_ = 0;
    for (const InvTask &t : iw) solve_flops_pq_ += 16.0 * t.n * t.n * t.n;
    for (const InvTask &t : id) solve_flops_dy_ += 8.0 * t.n * t.n * t.n;
  }
  qoff_irr_.upload(qo, st_);
  qsz_irr_.upload(qs, st_);
  pc_host_ = pc;
  sc_host_ = sc;
  sig_own_host_ = sig_own;
  GWGB_CUDA(cudaStreamSynchronize(st_));
}

// ---------------------------------------------------------------------------
// sliced (Ozaki) path: work lists of the six GEMM stages
// ---------------------------------------------------------------------------
namespace {

// Inclusive extent of the offsets of rows [0, M) of a row map.
void oz_rows_extent(const OzRows &m, int M, int64_t &lo, int64_t &hi) {
  const int64_t qmax = (M - 1) / m.d, rmax = std::min<int64_t>(m.d, M) - 1;
  lo = m.base + std::min<int64_t>(0, qmax * m.s1) + std::min<int64_t>(0, rmax * m.s0);
  hi = m.base + std::max<int64_t>(0, qmax * m.s1) + std::max<int64_t>(0, rmax * m.s0);
}

void oz_widen(int64_t &lo, int64_t &hi, int64_t step, int64_t count) {
  const int64_t e = (count - 1) * step;
  lo += std::min<int64_t>(0, e);
  hi += std::max<int64_t>(0, e);
}

// Every element that the tasks of descriptor d (nrep repetitions) read or
// write lies inside its buffers of na, nb, nc elements.
void oz_check(const OzDesc &d, int nrep, int64_t na, int64_t nb, int64_t nc, const char *what) {
  GWGB_REQUIRE(d.M >= 1 && d.N >= 1 && d.K >= 1 && nrep >= 1 && d.a.d >= 0 && d.b.d >= 0 && d.c.d >= 0 &&
                   d.cnd >= 1 && (d.a.d != 0 || d.aks == 1),
               GWGB_E_INVALID, std::string("internal work list out of bounds: empty sliced GEMM in ") + what);
  int64_t lo, hi;
  if (d.a.d != 0) {  // table-mapped rows are checked entry by entry where the table is built
    oz_rows_extent(d.a, d.M, lo, hi);
    oz_widen(lo, hi, d.aks, d.K);
    oz_widen(lo, hi, d.ra, nrep);
    check_range(lo, hi - lo + 1, na, what);
  }
  GWGB_REQUIRE(d.b.d != 0, GWGB_E_INVALID, std::string("internal work list: B rows must not be table-mapped in ") + what);
  oz_rows_extent(d.b, d.N, lo, hi);
  oz_widen(lo, hi, d.bks, d.K);
  oz_widen(lo, hi, d.rb, nrep);
  check_range(lo, hi - lo + 1, nb, what);
  if (d.c.d == 0) return;
  oz_rows_extent(d.c, d.M, lo, hi);
  const int64_t qmax = (d.N - 1) / d.cnd, rmax = std::min<int64_t>(d.cnd, d.N) - 1;
  lo += std::min<int64_t>(0, qmax * d.cn1) + std::min<int64_t>(0, rmax * d.cn0);
  hi += std::max<int64_t>(0, qmax * d.cn1) + std::max<int64_t>(0, rmax * d.cn0);
  oz_widen(lo, hi, d.rc, nrep);
  check_range(lo, hi - lo + 1, nc, what);
}

}  // namespace

bool Engine::build_oz_lists() {
  // Layouts (float-float, complex elements).  The contractions run in chunks of
  // output blocks (P0: output blocks (q_irr, iq); Sigma: AO blocks (k_irr, i1)
  // with their spins), each chunk over all tau (a block whose own buffers exceed
  // the budget: over tau ranges), so the final GEMMs (P0, Sigma) get full
  // 128-row tiles of (tau, row); a chunk's tau-dependent buffers are
  // sequences of tau slabs with one stride (z1t, zct, wct, uct elements per
  // tau), so one repetition offset serves every row of a packed GEMM.
  //   Z1[tau][pack][m][row]      row = (c, P, t) of the contributions sharing G2's block
  //   Zcat[tau][group][P][K]     K = (c, s, m, p) of the P0 output block (q_irr, iq)
  //   Vcat[group][Q][K]          = V_c[Q][p][m] at the same K (per chunk, or all chunks once per upload)
  //   W[tau][group][Q][col]      col = (c, j, n) of the chunk's contributions in the P~ block group
  //   U[tau][owner][j][K]        K = (c, Q, m) of the Sigma owner (k_irr, i1, s)
  //   VcatS[owner][i][K]         = Vt_c[Q][i][m] at the same K (per chunk, or all chunks once per upload)
  // Per-tau stages (Z1, Z, U) pack the chunk's contributions that share their
  // G-block operand (same block and spin) into one GEMM with a row table.
  const Lay &l = l_;
  const int ns = ns_, nts = nts_, half = nts / 2;
  const std::vector<P0Contrib> &pc = pc_host_;
  const std::vector<SigContrib> &sc = sc_host_;
  std::vector<OzDesc> ds;
  std::vector<OzTask> ts;
  std::vector<int64_t> rt;  // row table
  constexpr int REPG = 8;   // tau per task in the per-tau stages (Z, U)
  // narrow[id]: descriptor id runs on the CUDA-core kernel.  The choice uses a
  // width that does not depend on the chunking (width < 0: d.N), so chunked and
  // unchunked runs use the same arithmetic for every output element.
  std::vector<char> narrow_d;
  auto add = [&](const OzDesc &d, int nrep, int repg, int width = -1) {
    const int id = (int)ds.size();
    ds.push_back(d);
    narrow_d.push_back((width < 0 ? d.N : width) <= oz_simt_n_);
    const int mtn = (d.M + OZ_M - 1) / OZ_M, ntn = (d.N + OZ_NC - 1) / OZ_NC;
    GWGB_REQUIRE(mtn < 65536 && ntn < 65536, GWGB_E_UNSUPPORTED, "sliced GEMM too large");
    for (int r0 = 0; r0 < nrep; r0 += repg)
      for (int mt = 0; mt < mtn; ++mt)
        for (int nt = 0; nt < ntn; ++nt) ts.push_back({id, r0, std::min(repg, nrep - r0), (mt << 16) | nt});
  };
  // tasks of one stage (appended since t0): the tensor-core tasks, then the
  // narrow ones (at most oz_simt_n_ output columns) for the CUDA-core kernel,
  // each heaviest first; one launch per kind.  The last launch carries `last`.
  auto narrow = [&](const OzTask &t) { return narrow_d[t.desc] != 0; };
  int cur_stage = 0;  // gwgb_launch_stat.stage of the launches being built
  auto stage = [&](std::vector<OzLaunch> &v, size_t t0, int a, int b, int c, bool part = false,
                   const OzLaunch *last = nullptr) {
    auto cost = [&](const OzTask &t) { return (int64_t)t.nrep * ds[t.desc].K; };
    std::stable_sort(ts.begin() + t0, ts.end(), [&](const OzTask &x, const OzTask &y) {
      const bool nx = narrow(x), ny = narrow(y);
      return nx != ny ? ny : cost(x) > cost(y);
    });
    const size_t t1 = std::find_if(ts.begin() + t0, ts.end(), narrow) - ts.begin();
    const size_t n0 = v.size();
    for (int k = 0; k < 2; ++k) {
      const size_t lo = k ? t1 : t0, hi = k ? ts.size() : t1;
      if (hi == lo) continue;
      OzLaunch l{(int64_t)lo, (int64_t)(hi - lo), a, b, c};
      l.simt = k == 1;
      l.part = part;
      l.stage = cur_stage;
      for (size_t t = lo; t < hi; ++t) {  // algorithmic FLOPs; tcgen05 MMA FLOPs or FP32 instructions
        const OzTask &tk = ts[t];
        const OzDesc &d = ds[tk.desc];
        const int Mt = std::min(OZ_M, d.M - (tk.mtnt >> 16) * OZ_M), Nt = std::min(OZ_NC, d.N - (tk.mtnt & 0xffff) * OZ_NC);
        const double cmac = (double)Mt * Nt * d.K * tk.nrep;
        l.flops += 8.0 * cmac;
        if (l.simt) {
          l.ops += 48.0 * cmac;
        } else {
          const int ksteps = (d.K / OZ_KR) * 2 + ((d.K % OZ_KR) + 7) / 8;  // MMA K steps of 8 complex
          l.ops += 10.0 * 2.0 * OZ_M * (16.0 * ((Nt + 7) / 8)) * 16.0 * ksteps * tk.nrep;
        }
      }
      v.push_back(l);
    }
    if (last && v.size() > n0) {
      v.back().r0 = last->r0;
      v.back().nr = last->nr;
      v.back().scale = last->scale;
      v.back().red_bytes = last->red_bytes;
      v.back().red_ny = last->red_ny;
    }
  };
  // Final GEMMs (P0, Sigma) in K slices: each slice writes an FP64 partial block
  // [slice][rows][cols] to ozPart_; the slices are summed in order afterwards
  // (reduce_slices_kernel), so the result does not depend on the launch order.
  // The slice count depends on the block alone (about two waves of CTAs for
  // that block, at least 32 rounds of K per slice), so results do not depend on
  // how blocks are grouped into chunks.
  std::vector<RedTask> red;
  // mfull: rows of the block over all tau (the slice count must not depend on the tau chunking)
  struct Fin { OzDesc d; int64_t out; int32_t ostride, nt, elems, mfull; };
  auto final_stage = [&](std::vector<OzLaunch> &v, const std::vector<Fin> &fins, int a, int b, int c, double scale,
                         int64_t na, int64_t nb, int64_t nout, const char *what) {
    const size_t t0 = ts.size(), r0 = red.size();
    int64_t part = 0;
    for (const Fin &f : fins) {
      const int64_t tiles = (int64_t)((f.mfull + OZ_M - 1) / OZ_M) * ((f.d.N + OZ_NC - 1) / OZ_NC);
      const int64_t want = (2 * (int64_t)std::max(1, nsm_) + tiles - 1) / tiles;
      const int nk16 = (f.d.K + OZ_KR - 1) / OZ_KR;
      const int nsl = (int)std::max<int64_t>(1, std::min<int64_t>(want, nk16 / 32));
      const int per = (nk16 + nsl - 1) / nsl * OZ_KR;
      const int64_t mn = (int64_t)f.d.M * f.d.N;
      int used = 0;
      for (int k0 = 0; k0 < f.d.K; k0 += per, ++used) {
        OzDesc d = f.d;
        d.a.base += k0;
        d.b.base += k0;
        d.K = std::min(per, f.d.K - k0);
        d.c = {part + used * mn, f.elems, 1, f.d.c.d};
        d.alpha = 1.0;
        d.flags |= OZ_OUT_F64;
        oz_check(d, 1, na, nb, (int64_t)1 << 62, what);
        add(d, 1, 1);
      }
      red.push_back({part, f.out, f.ostride, f.elems, 0, f.nt, used, 0});
      check_range(f.out, (int64_t)(f.nt - 1) * f.ostride + f.elems, nout, what);
      part += used * mn;
    }
    oz_part_elems_ = std::max(oz_part_elems_, part);
    OzLaunch red_info{0, 0, a, b, c};
    red_info.r0 = (int64_t)r0;
    red_info.nr = (int64_t)(red.size() - r0);
    red_info.scale = scale;
    int64_t maxn = 1;
    for (size_t r = r0; r < red.size(); ++r) {  // partials read, output written
      red_info.red_bytes += 16.0 * red[r].nt * red[r].elems * (red[r].nslice + 1);
      maxn = std::max<int64_t>(maxn, (int64_t)red[r].nt * red[r].elems);
    }
    // enough CTAs for about four waves of 256-thread blocks, none with under 1024 elements
    const int64_t nblk = std::max<int64_t>(1, (int64_t)(red.size() - r0));
    const int64_t want = (4 * 8 * (int64_t)std::max(1, nsm_) + nblk - 1) / nblk;
    red_info.red_ny = (int)std::max<int64_t>(1, std::min<int64_t>({want, (maxn + 1023) / 1024, 4096}));
    stage(v, t0, a, b, c, true, &red_info);
  };
  // Row-table checks: every entry (plus the row's K extent and reps) inside the buffer.
  auto check_tab = [&](int64_t base, int M, int64_t klen, int64_t rep, int nrep, int64_t size, const char *what) {
    for (int r = 0; r < M; ++r) {
      int64_t lo = rt[base + r], hi = lo + klen - 1;
      oz_widen(lo, hi, rep, nrep);
      check_range(lo, hi - lo + 1, size, what);
    }
  };
  oz_p0_.clear();
  oz_sig_.clear();
  oz_part_elems_ = 1;
  const int64_t gsz = (int64_t)Gall_.n, psz = (int64_t)Pall_.n, ssz = (int64_t)nts * ns * l.flat_ao;
  const double pref = -1.0 / l.nk * (ns == 1 ? 2.0 : 1.0);  // cugw_qkpt_block.cu:210, cugw_solver_block.cpp:303

  // ---- P0 -------------------------------------------------------------------
  // Operand builds (copies of V / Vt blocks): one launch per chunk and buffer, or
  // a launch in oz_static_ (once per upload) when the contraction has one chunk.
  std::vector<OzPerm> perms;
  oz_static_.clear();
  auto perm_launch = [&](std::vector<OzLaunch> &v, size_t p0, int src, int dst, bool once) {
    if (perms.size() == p0) return;
    OzLaunch l{(int64_t)p0, (int64_t)(perms.size() - p0), src, src, dst};
    l.perm = true;
    l.stage = cur_stage;
    for (size_t t = p0; t < perms.size(); ++t) l.red_bytes += 32.0 * perms[t].X * perms[t].Y * perms[t].Z;
    (once ? oz_static_ : v).push_back(l);
  };
  struct PG { int64_t voff; int zld; };  // Vcat offset (chunk-local) and row length of a P0 group
  std::vector<PG> pg;
  std::vector<int> zcol(pc.size() * ns), cgrp(pc.size());
  for (size_t gi = 0; gi < p0_groups_.size(); ++gi) {
    const P0Group &g = p0_groups_[gi];
    int zld = 0;
    for (int c = g.c0; c < g.c1; ++c) {
      cgrp[c] = (int)gi;
      for (int sp = 0; sp < ns; ++sp) {
        zcol[c * ns + sp] = zld;
        zld += pc[c].b1 * pc[c].b2;
      }
    }
    pg.push_back({0, zld});
  }
  // chunks of output blocks: Z1, Zcat, Vcat and V blocks of a chunk (all nts/2 tau) within
  // the budget: 1/oz_div_ of the memory free now (after V), at most GWGB_TC_CHUNK_MB
  // when that is given, at least 64 MB.  Every buffer is sized to its largest chunk and
  // the P0 and Sigma buffers coexist; the caller halves the budget until they fit.
  int64_t budget;  // complex float-float elements
  {
    size_t free_b = 0, total_b = 0;
    GWGB_CUDA(cudaMemGetInfo(&free_b, &total_b));
    const int64_t by_free = std::max<int64_t>(64ll << 20, (int64_t)(free_b / oz_div_));
    budget = std::max<int64_t>(1, (tc_chunk_env_ ? std::min<int64_t>(tc_chunk_bytes_, by_free) : by_free) / 16);
  }
  // The concatenated operands of every chunk are kept (built once per upload) when
  // together they take at most a quarter of the free memory; otherwise each chunk
  // builds its own in the launch list.
  bool persist;
  {
    int64_t tot = 0;
    for (size_t gi = 0; gi < p0_groups_.size(); ++gi) tot += 2 * (int64_t)p0_groups_[gi].qb * pg[gi].zld;
    for (const SigContrib &x : sc) tot += 2 * (int64_t)x.qb * x.b2 * 64;  // Bcat + VcatS, AO blocks <= 64
    size_t free_b = 0, total_b = 0;
    GWGB_CUDA(cudaMemGetInfo(&free_b, &total_b));
    persist = tot * 16 <= (int64_t)(free_b / 4);
  }
  int64_t vcat_base = 0, vz_base = 0, bcat_base = 0, vcats_base = 0;  // persistent: each chunk's offset
  // persistent: where a block's operand copy already is (tau chunks of one block share it)
  std::vector<int64_t> vcat_at(p0_groups_.size(), -1), vz_at(pc.size(), -1);
  std::map<std::pair<int, int>, int64_t> bcat_at, vcats_at;
  // A group whose own need is above the budget gets chunks of its own over tau ranges.
  struct Chunk { int first, second, t0, t1; };  // output blocks [first, second), tau [t0, t1)
  std::vector<Chunk> pchunks;
  {
    auto need = [&](size_t g, int nt) {  // Z1 and Zcat per tau, Vcat and V blocks once
      return (2 * (int64_t)nt + 2) * p0_groups_[g].qb * pg[g].zld;
    };
    for (size_t g0 = 0; g0 < p0_groups_.size();) {
      if (need(g0, half) > budget) {
        const int64_t per = 2 * (int64_t)p0_groups_[g0].qb * pg[g0].zld;
        const int nt = (int)std::max<int64_t>(1, std::min<int64_t>(half, (budget - per) / per));
        for (int t0 = 0; t0 < half; t0 += nt) pchunks.push_back({(int)g0, (int)g0 + 1, t0, std::min(half, t0 + nt)});
        ++g0;
        continue;
      }
      size_t g1 = g0;
      int64_t tot = 0;
      while (g1 < p0_groups_.size() && need(g1, half) <= budget && (g1 == g0 || tot + need(g1, half) <= budget))
        tot += need(g1++, half);
      pchunks.push_back({(int)g0, (int)g1, 0, half});
      g0 = g1;
    }
  }
  oz_z1_elems_ = oz_zcat_elems_ = oz_vcat_elems_ = oz_vz_elems_ = 1;
  struct PackRow { int c; int64_t pos; };
  for (const auto &ch : pchunks) {
    const int t0 = ch.t0, ntc = ch.t1 - ch.t0;  // the chunk's tau range
    {  // Vcat of the chunk's groups: Vcat[Q][zcol + m b1 + p] = V_c[Q][p][m]
      const size_t p0 = perms.size();
      int64_t voff = persist ? vcat_base : 0;
      for (int gi = ch.first; gi < ch.second; ++gi) {
        const P0Group &g = p0_groups_[gi];
        if (persist && vcat_at[gi] >= 0) {
          pg[gi].voff = vcat_at[gi];
          continue;
        }
        pg[gi].voff = voff;
        vcat_at[gi] = voff;
        for (int c = g.c0; c < g.c1; ++c)
          for (int sp = 0; sp < ns; ++sp)
            perms.push_back({pc[c].v, voff + zcol[c * ns + sp], pg[gi].zld, 1, pc[c].b1, g.qb, pc[c].b1, pc[c].b2, 0});
        voff += (int64_t)g.qb * pg[gi].zld;
      }
      oz_vcat_elems_ = std::max(oz_vcat_elems_, voff);
      for (size_t t = p0; t < perms.size(); ++t) {
        const OzPerm &x = perms[t];
        check_range(x.src, (int64_t)x.X * x.Y * x.Z, l.flat_V, "sliced Vcat source");
        check_range(x.dst, (x.X - 1) * x.dx + (x.Y - 1) * x.dy + (x.Z - 1) * x.dz + 1, voff, "sliced Vcat");
      }
      if (persist) vcat_base = voff;
      cur_stage = 2;
      perm_launch(oz_p0_, p0, OZB_V, OZB_VCAT, persist || pchunks.size() == 1);
    }
    std::vector<int64_t> vz(pc.size(), -1);  // the chunk's V blocks in float-float (the Z1 stage's A rows)
    int64_t vz_elems = persist ? vz_base : 0;
    {
      const size_t p0 = perms.size();
      int64_t &off = vz_elems;
      for (int gi = ch.first; gi < ch.second; ++gi)
        for (int c = p0_groups_[gi].c0; c < p0_groups_[gi].c1; ++c) {
          const int qb = p0_groups_[gi].qb, b1 = pc[c].b1, b2 = pc[c].b2;
          if (persist && vz_at[c] >= 0) {
            vz[c] = vz_at[c];
            continue;
          }
          vz[c] = vz_at[c] = off;
          perms.push_back({pc[c].v, off, (int64_t)b1 * b2, b2, 1, qb, b1, b2, 0});
          check_range(pc[c].v, (int64_t)qb * b1 * b2, l.flat_V, "sliced V block source");
          off += (int64_t)qb * b1 * b2;
        }
      oz_vz_elems_ = std::max(oz_vz_elems_, off);
      if (persist) vz_base = off;
      cur_stage = 0;
      perm_launch(oz_p0_, p0, OZB_V, OZB_VZ, persist || pchunks.size() == 1);
    }
    // chunk-local per-tau layouts
    std::vector<int64_t> zc(p0_groups_.size(), 0);
    int64_t zct = 0;
    for (int gi = ch.first; gi < ch.second; ++gi) {
      zc[gi] = zct;
      zct += (int64_t)p0_groups_[gi].qb * pg[gi].zld;
    }
    std::map<std::pair<int64_t, int>, std::vector<PackRow>> z1p, zp;
    for (int gi = ch.first; gi < ch.second; ++gi)
      for (int c = p0_groups_[gi].c0; c < p0_groups_[gi].c1; ++c)
        for (int sp = 0; sp < ns; ++sp) {
          auto &v = z1p[{pc[c].gb, sp}];
          const int64_t pos =
              v.empty() ? 0 : v.back().pos + (int64_t)p0_groups_[cgrp[v.back().c]].qb * pc[v.back().c].b1;
          v.push_back({c, pos});
          zp[{pc[c].ga, sp}].push_back({c, 0});
        }
    std::map<int, int64_t> z1pack, z1mp, z1pos;  // keyed by c * ns + s
    int64_t z1t = 0;
    for (auto &kv : z1p) {
      const auto &v = kv.second;
      const int64_t mp = v.back().pos + (int64_t)p0_groups_[cgrp[v.back().c]].qb * pc[v.back().c].b1;
      for (const PackRow &x : v) {
        const int k = x.c * ns + kv.first.second;
        z1pack[k] = z1t;
        z1mp[k] = mp;
        z1pos[k] = x.pos;
      }
      z1t += mp * pc[v[0].c].b2;
    }
    const int64_t z1_elems = z1t * ntc, zcat_elems = zct * ntc;
    oz_z1_elems_ = std::max(oz_z1_elems_, z1_elems);
    oz_zcat_elems_ = std::max(oz_zcat_elems_, zcat_elems);
    size_t s0 = ts.size();
    for (auto &kv : z1p) {  // Z1[tau][m][(c,P,t)] = sum_n conj(V_c[P][t][n]) G2(tau)[m][n]
      const int sp = kv.first.second;
      const auto &v = kv.second;
      const P0Contrib &c0 = pc[v[0].c];
      const int b2 = c0.b2, k0 = v[0].c * ns + sp;
      const int64_t tab = (int64_t)rt.size();
      for (const PackRow &x : v) {
        const P0Contrib &cb = pc[x.c];
        const int qb = p0_groups_[cgrp[x.c]].qb;
        for (int P = 0; P < qb; ++P)
          for (int t = 0; t < cb.b1; ++t) rt.push_back(vz[x.c] + ((int64_t)P * cb.b1 + t) * b2);
      }
      OzDesc d{};
      d.M = (int)(rt.size() - tab);
      d.a = {tab, 0, 0, 0};
      d.b = {c0.gb + ((int64_t)t0 * ns + sp) * c0.sb, (int64_t)ns * c0.sb, b2, b2};  // G2(tau) rows (tau, m)
      d.c = {z1pack[k0], 1, 0, 1};
      d.cn1 = z1t;
      d.cn0 = (int32_t)z1mp[k0];
      d.cnd = b2;
      d.aks = d.bks = 1;
      d.N = ntc * b2;
      d.K = b2;
      d.flags = OZ_CONJ_A;
      check_tab(tab, d.M, b2, 0, 1, vz_elems, "P0 stage Z1 (V rows)");
      oz_check(d, 1, vz_elems, gsz, z1_elems, "P0 stage Z1");
      add(d, 1, 1, half * b2);  // routed by the width over all tau (every tau chunk the same way)
    }
    cur_stage = 0;
    stage(oz_p0_, s0, OZB_VZ, OZB_G, OZB_Z1);
    s0 = ts.size();
    for (auto &kv : zp) {  // Zcat[tau][P][K = (c,s,m,p)] = sum_t G1(beta-tau)[t][p] Z1[tau][m][(c,P,t)]
      const int sp = kv.first.second;
      const auto &v = kv.second;
      const P0Contrib &c0 = pc[v[0].c];
      const int b1 = c0.b1;
      const int64_t taba = (int64_t)rt.size();
      for (const PackRow &x : v) {
        const P0Contrib &cb = pc[x.c];
        const int qb = p0_groups_[cgrp[x.c]].qb, k = x.c * ns + sp;
        for (int P = 0; P < qb; ++P)
          for (int m = 0; m < cb.b2; ++m) rt.push_back(z1pack[k] + m * z1mp[k] + z1pos[k] + (int64_t)P * b1);
      }
      const int64_t tabc = (int64_t)rt.size();
      for (const PackRow &x : v) {
        const P0Contrib &cb = pc[x.c];
        const int gi = cgrp[x.c], qb = p0_groups_[gi].qb, k = x.c * ns + sp;
        for (int P = 0; P < qb; ++P)
          for (int m = 0; m < cb.b2; ++m) rt.push_back(zc[gi] + (int64_t)P * pg[gi].zld + zcol[k] + (int64_t)m * b1);
      }
      OzDesc d{};
      d.M = (int)(tabc - taba);
      d.a = {taba, 0, 0, 0};
      d.ra = z1t;
      d.b = {c0.ga + ((int64_t)(nts - 1 - t0) * ns + sp) * c0.sa, 1, 0, 1};  // G1(beta - tau)
      d.bks = b1;
      d.rb = -(int64_t)ns * c0.sa;
      d.c = {tabc, 0, 0, 0};
      d.rc = zct;
      d.cn1 = 1;
      d.cnd = 1;
      d.aks = 1;
      d.N = b1;
      d.K = b1;
      check_tab(taba, d.M, b1, z1t, ntc, z1_elems, "P0 stage Z (Z1 rows)");
      check_tab(tabc, d.M, b1, zct, ntc, zcat_elems, "P0 stage Z (Zcat rows)");
      oz_check(d, ntc, z1_elems, gsz, zcat_elems, "P0 stage Z");
      add(d, ntc, REPG);
    }
    cur_stage = 1;
    stage(oz_p0_, s0, OZB_Z1, OZB_G, OZB_ZCAT);
    std::vector<Fin> fins;
    for (int gi = ch.first; gi < ch.second; ++gi) {  // P0[Q][P] = sum_K Zcat[(tau,P)][K] Vcat[Q][K]
      const P0Group &g = p0_groups_[gi];
      if (g.c1 == g.c0) continue;
      OzDesc d{};
      d.a = {zc[gi], zct, pg[gi].zld, g.qb};
      d.b = {pg[gi].voff, pg[gi].zld, 0, 1};
      d.c = {0, 0, 1, g.qb};  // partial [slice][(tau, P)][Q]: rows (tau, P), column Q at Q * qb
      d.cn1 = g.qb;
      d.cnd = 1;
      d.aks = d.bks = 1;
      d.M = ntc * g.qb;
      d.N = g.qb;
      d.K = pg[gi].zld;
      oz_check(d, 1, zcat_elems, oz_vcat_elems_, (int64_t)1 << 62, "P0 stage P0");
      fins.push_back({d, g.pout + (int64_t)t0 * g.pstride, g.pstride, ntc, g.qb * g.qb, half * g.qb});
    }
    cur_stage = 2;
    final_stage(oz_p0_, fins, OZB_ZCAT, OZB_VCAT, OZB_P0, pref, zcat_elems, oz_vcat_elems_, psz, "P0 stage P0");
  }

  // ---- Sigma ----------------------------------------------------------------
  // Bcat per P~ block group, columns in contribution order (so the columns of a
  // chunk of AO-block owners are contiguous in every group); chunk-local copies
  struct SG { int qb, ncol; };
  std::vector<SG> sg;
  std::vector<int> cgroup(sc.size(), -1), ccol(sc.size(), 0);
  std::vector<std::vector<int>> gcs;  // contributions of each group (increasing)
  for (const auto &grp : sig_groups_) {
    const std::vector<int> &cs = grp.second;
    const int qb = sc[cs[0]].qb;
    int ncol = 0;
    for (int c : cs) {
      cgroup[c] = (int)sg.size();
      ccol[c] = ncol;
      ncol += sig_b1_[c] * sc[c].b2;
    }
    sg.push_back({qb, ncol});
    gcs.push_back(cs);
  }
  // AO-block owners (k_irr, i1): the owners of their spins share (c0, c1)
  std::vector<int> ucol(sc.size(), 0);
  std::map<std::pair<int, int>, int> uldk;  // (c0, c1) -> row length of U and VcatS
  std::vector<std::pair<int, int>> aoo;     // distinct (c0, c1) in owner order
  std::map<std::pair<int, int>, int> aoidx; // (c0, c1) -> index in aoo
  std::map<std::pair<int, int>, int> aon;   // (c0, c1) -> block size (rows of VcatS)
  for (size_t oi = 0; oi < sig_own_host_.size(); ++oi) {
    const Owner &o = sig_own_host_[oi];
    const auto key = std::make_pair(o.c0, o.c1);
    if (uldk.count(key)) continue;
    int uld = 0;
    for (int c = o.c0; c < o.c1; ++c) {
      ucol[c] = uld;
      uld += sc[c].qb * sc[c].b2;
    }
    uldk[key] = uld;
    aon[key] = o.n;
    aoidx[key] = (int)aoo.size();
    aoo.push_back(key);
  }
  // chunks of AO-block owners: W and U of a chunk (all nts tau) and its Bcat and
  // VcatS within the budget
  // An owner whose own need is above the budget gets chunks of its own over tau ranges.
  auto ao_w = [&](const std::pair<int, int> &key) {
    int64_t w = 0;
    for (int c = key.first; c < key.second; ++c) w += (int64_t)sc[c].qb * sig_b1_[c] * sc[c].b2;
    return w;
  };
  auto ao_need = [&](const std::pair<int, int> &key, int nt) {  // W and U per tau, Bcat and VcatS once
    const int64_t w = ao_w(key);
    return (1 + ns) * w * nt + w + (int64_t)aon[key] * uldk[key];
  };
  std::vector<Chunk> schunks;  // ranges of aoo, tau ranges
  for (size_t a0 = 0; a0 < aoo.size();) {
    if (ao_need(aoo[a0], nts) > budget) {
      const int64_t per = (1 + ns) * ao_w(aoo[a0]), fixed = ao_need(aoo[a0], 0);
      const int nt = (int)std::max<int64_t>(1, std::min<int64_t>(nts, (budget - fixed) / per));
      for (int t0 = 0; t0 < nts; t0 += nt) schunks.push_back({(int)a0, (int)a0 + 1, t0, std::min(nts, t0 + nt)});
      ++a0;
      continue;
    }
    size_t a1 = a0;
    int64_t tot = 0;
    while (a1 < aoo.size() && ao_need(aoo[a1], nts) <= budget && (a1 == a0 || tot + ao_need(aoo[a1], nts) <= budget))
      tot += ao_need(aoo[a1++], nts);
    schunks.push_back({(int)a0, (int)a1, 0, nts});
    a0 = a1;
  }
  oz_w_elems_ = oz_u_elems_ = oz_bcat_elems_ = oz_vcats_elems_ = 1;
  for (const auto &ch : schunks) {
    const int t0 = ch.t0, ntc = ch.t1 - ch.t0;                           // the chunk's tau range
    const int cA = aoo[ch.first].first, cB = aoo[ch.second - 1].second;  // contributions [cA, cB)
    // W: per group, the chunk's columns (contiguous: contributions in [cA, cB)); the
    // chunk's Bcat holds those columns, group after group: Bcat[col][P] = conj(Vt_c[P][j][n])
    struct WG { int g, col0, ncol; int64_t wc, boff; };
    std::vector<WG> wg;
    std::vector<int> wgi(sg.size(), -1);
    int64_t wct = 0, boff = persist ? bcat_base : 0;
    const size_t pb0 = perms.size();
    for (size_t gi = 0; gi < sg.size(); ++gi) {
      int col0 = -1, ncol = 0;
      for (int c : gcs[gi])
        if (c >= cA && c < cB) {
          if (col0 < 0) col0 = ccol[c];
          ncol += sig_b1_[c] * sc[c].b2;
        }
      if (ncol == 0) continue;
      const int qb = sg[gi].qb;
      int64_t at = boff;
      auto hit = bcat_at.find({(int)gi, cA});
      if (persist && hit != bcat_at.end()) {
        at = hit->second;
      } else {
        for (int c : gcs[gi])
          if (c >= cA && c < cB)
            perms.push_back({sc[c].v, boff + (int64_t)(ccol[c] - col0) * qb, 1, (int64_t)sc[c].b2 * qb, qb, qb,
                             sig_b1_[c], sc[c].b2, 1});
        bcat_at[{(int)gi, cA}] = boff;
        boff += (int64_t)qb * ncol;
      }
      wgi[gi] = (int)wg.size();
      wg.push_back({(int)gi, col0, ncol, wct, at});
      wct += (int64_t)qb * ncol;
    }
    oz_bcat_elems_ = std::max(oz_bcat_elems_, boff);
    for (size_t t = pb0; t < perms.size(); ++t) {
      const OzPerm &x = perms[t];
      check_range(x.src, (int64_t)x.X * x.Y * x.Z, (int64_t)Vt_.n, "sliced Bcat source");
      check_range(x.dst, (x.X - 1) * x.dx + (x.Y - 1) * x.dy + (x.Z - 1) * x.dz + 1, boff, "sliced Bcat");
    }
    if (persist) bcat_base = boff;
    cur_stage = 3;
    perm_launch(oz_sig_, pb0, OZB_VT, OZB_BCAT, persist || schunks.size() == 1);
    // VcatS of the chunk's owner blocks: VcatS[i][ucol + Q b2 + n] = Vt_c[Q][i][n]
    const size_t ps0 = perms.size();
    std::map<std::pair<int, int>, std::pair<int64_t, int>> vs;  // (c0, c1) -> (VcatS offset, uld)
    int64_t vsoff = persist ? vcats_base : 0;
    for (int ai = ch.first; ai < ch.second; ++ai) {
      const auto key = aoo[ai];
      const int uld = uldk[key];
      auto hit = vcats_at.find(key);
      if (persist && hit != vcats_at.end()) {
        vs[key] = {hit->second, uld};
        continue;
      }
      vs[key] = {vsoff, uld};
      vcats_at[key] = vsoff;
      for (int c = key.first; c < key.second; ++c)
        perms.push_back({sc[c].v, vsoff + ucol[c], sc[c].b2, uld, 1, sc[c].qb, sig_b1_[c], sc[c].b2, 0});
      vsoff += (int64_t)aon[key] * uld;
    }
    oz_vcats_elems_ = std::max(oz_vcats_elems_, vsoff);
    for (size_t t = ps0; t < perms.size(); ++t) {
      const OzPerm &x = perms[t];
      check_range(x.src, (int64_t)x.X * x.Y * x.Z, (int64_t)Vt_.n, "sliced VcatS source");
      check_range(x.dst, (x.X - 1) * x.dx + (x.Y - 1) * x.dy + (x.Z - 1) * x.dz + 1, vsoff, "sliced VcatS");
    }
    if (persist) vcats_base = vsoff;
    cur_stage = 5;
    perm_launch(oz_sig_, ps0, OZB_VT, OZB_VCATS, persist || schunks.size() == 1);
    // U: the chunk's owners (all spins)
    std::vector<int64_t> uoff(sig_own_host_.size(), -1);
    int64_t uct = 0;
    for (size_t oi = 0; oi < sig_own_host_.size(); ++oi) {
      const Owner &o = sig_own_host_[oi];
      const int ai = aoidx[std::make_pair(o.c0, o.c1)];
      if (ai < ch.first || ai >= ch.second) continue;
      uoff[oi] = uct;
      uct += (int64_t)o.n * vs[std::make_pair(o.c0, o.c1)].second;
    }
    const int64_t w_elems = std::max<int64_t>(1, wct * ntc), u_elems = std::max<int64_t>(1, uct * ntc);
    oz_w_elems_ = std::max(oz_w_elems_, w_elems);
    oz_u_elems_ = std::max(oz_u_elems_, u_elems);
    size_t s0 = ts.size();
    for (const WG &w : wg) {  // W[tau][Q][(c,j,n)] = sum_P op(P~(tau))[Q][P] conj(Vt_c[P][j][n])
      const SigContrib &c0 = sc[gcs[w.g][0]];
      const int qb = c0.qb;
      OzDesc d{};
      d.a = {c0.pq + (int64_t)t0 * c0.pstride, c0.pstride, qb, qb};  // P~ rows (tau, Q) of the tau range
      d.b = {w.boff, qb, 0, 1};  // the chunk's Bcat columns of this group
      d.c = {w.wc, wct, w.ncol, qb};
      d.cn1 = 1;
      d.cnd = 1;
      d.aks = d.bks = 1;
      d.M = ntc * qb;
      d.N = w.ncol;
      d.K = qb;
      d.flags = c0.pconj ? OZ_CONJ_A : 0;
      oz_check(d, 1, psz, oz_bcat_elems_, w_elems, "Sigma stage W");
      add(d, 1, 1, sg[w.g].ncol);  // routed by the group's full width (every chunk the same way)
    }
    cur_stage = 3;
    stage(oz_sig_, s0, OZB_P, OZB_BCAT, OZB_W);
    s0 = ts.size();
    // U packs: (G2 block, spin) -> [(owner, contribution)]
    std::map<std::pair<int64_t, int>, std::vector<std::pair<int, int>>> up;
    for (size_t oi = 0; oi < sig_own_host_.size(); ++oi) {
      if (uoff[oi] < 0) continue;
      const Owner &o = sig_own_host_[oi];
      for (int c = o.c0; c < o.c1; ++c) up[{sc[c].gb, o.s}].push_back({(int)oi, c});
    }
    for (auto &kv : up) {  // U[tau][j][(c,Q,m)] = sum_n W[tau][Q][(c,j,n)] G2(tau)[m][n]
      const int sp = kv.first.second;
      const auto &v = kv.second;
      const SigContrib &c0 = sc[v[0].second];
      const int b2 = c0.b2;
      const int64_t taba = (int64_t)rt.size();
      for (const auto &x : v) {
        const int c = x.second, b1 = sig_b1_[c];
        const WG &w = wg[wgi[cgroup[c]]];
        for (int Q = 0; Q < sc[c].qb; ++Q)
          for (int j = 0; j < b1; ++j)
            rt.push_back(w.wc + (int64_t)Q * w.ncol + (ccol[c] - w.col0) + (int64_t)j * b2);
      }
      const int64_t tabc = (int64_t)rt.size();
      for (const auto &x : v) {
        const int c = x.second, b1 = sig_b1_[c];
        const Owner &o = sig_own_host_[x.first];
        const int uld = vs[std::make_pair(o.c0, o.c1)].second;
        for (int Q = 0; Q < sc[c].qb; ++Q)
          for (int j = 0; j < b1; ++j) rt.push_back(uoff[x.first] + ucol[c] + (int64_t)Q * b2 + (int64_t)j * uld);
      }
      OzDesc d{};
      d.M = (int)(tabc - taba);
      d.a = {taba, 0, 0, 0};
      d.ra = wct;
      d.b = {c0.gb + ((int64_t)t0 * ns + sp) * c0.sb, b2, 0, 1};  // G2(tau), tau from t0
      d.rb = (int64_t)ns * c0.sb;
      d.c = {tabc, 0, 0, 0};
      d.rc = uct;
      d.cn1 = 1;
      d.cnd = 1;
      d.aks = d.bks = 1;
      d.N = b2;
      d.K = b2;
      check_tab(taba, d.M, b2, wct, ntc, w_elems, "Sigma stage U (W rows)");
      check_tab(tabc, d.M, b2, uct, ntc, u_elems, "Sigma stage U (U rows)");
      oz_check(d, ntc, w_elems, gsz, u_elems, "Sigma stage U");
      add(d, ntc, REPG);
    }
    cur_stage = 4;
    stage(oz_sig_, s0, OZB_W, OZB_G, OZB_U);
    std::vector<Fin> fins;
    for (size_t oi = 0; oi < sig_own_host_.size(); ++oi) {  // Sigma[i][j] = sum_K U[(tau,j)][K] VcatS[i][K]
      if (uoff[oi] < 0) continue;
      const Owner &o = sig_own_host_[oi];
      const auto &v = vs[std::make_pair(o.c0, o.c1)];
      if (v.second == 0) continue;
      OzDesc d{};
      d.a = {uoff[oi], uct, v.second, o.n};
      d.b = {v.first, v.second, 0, 1};
      d.c = {0, 0, 1, o.n};  // partial [slice][(tau, j)][i]: rows (tau, j), column i at i * b1
      d.cn1 = o.n;
      d.cnd = 1;
      d.aks = d.bks = 1;
      d.M = ntc * o.n;
      d.N = o.n;
      d.K = v.second;
      oz_check(d, 1, u_elems, oz_vcats_elems_, (int64_t)1 << 62, "Sigma stage Sigma");
      fins.push_back({d, o.out + (int64_t)t0 * o.ostride, o.ostride, ntc, o.n * o.n, nts * o.n});
    }
    cur_stage = 5;
    final_stage(oz_sig_, fins, OZB_U, OZB_VCATS, OZB_SIG, -1.0 / l.nk, u_elems, oz_vcats_elems_, ssz,
                "Sigma stage Sigma");
  }
  GWGB_REQUIRE(ts.size() < (size_t)INT32_MAX, GWGB_E_UNSUPPORTED, "too many sliced GEMM tasks");
  {  // buffers and lists within 85% of the free memory, or a smaller budget
    const int64_t bufs = 16 * (oz_z1_elems_ + oz_zcat_elems_ + oz_w_elems_ + oz_u_elems_ + oz_vcat_elems_ +
                               oz_bcat_elems_ + oz_vcats_elems_ + oz_vz_elems_ + oz_part_elems_ +
                               (int64_t)(Gall_.n + Pall_.n)) +
                         (int64_t)(ds.size() * sizeof(OzDesc) + ts.size() * sizeof(OzTask) + rt.size() * 8);
    size_t free_b = 0, total_b = 0;
    GWGB_CUDA(cudaMemGetInfo(&free_b, &total_b));
    if (bufs > (int64_t)(0.85 * (double)free_b) && oz_div_ < 256) return false;
  }
  {
    const int64_t lists = (int64_t)(ds.size() * sizeof(OzDesc) + ts.size() * sizeof(OzTask) + rt.size() * 8 +
                                    perms.size() * sizeof(OzPerm) + red.size() * sizeof(RedTask));
    size_t free_b = 0, total_b = 0;
    GWGB_CUDA(cudaMemGetInfo(&free_b, &total_b));
    GWGB_REQUIRE(lists + (256ll << 20) <= (int64_t)free_b, GWGB_E_UNSUPPORTED,
                 "sliced-precision work lists need " + std::to_string(lists >> 20) + " MB (row tables " +
                     std::to_string((rt.size() * 8) >> 20) + " MB, tasks " +
                     std::to_string((ts.size() * sizeof(OzTask)) >> 20) + " MB), " + std::to_string(free_b >> 20) +
                     " MB free");
  }
  oz_descs_.upload(ds, st_);
  oz_tasks_.upload(ts, st_);
  oz_rowtab_.upload(rt.empty() ? std::vector<int64_t>(1, 0) : rt, st_);
  for (const RedTask &r : red) check_range(r.part, (int64_t)r.nslice * r.nt * r.elems, oz_part_elems_, "sliced partials");
  oz_red_.upload(red.empty() ? std::vector<RedTask>(1, RedTask{}) : red, st_);
  oz_perm_.upload(perms.empty() ? std::vector<OzPerm>(1, OzPerm{}) : perms, st_);
  GWGB_CUDA(cudaStreamSynchronize(st_));
  lt_build();
  oz_built_ = true;
  return true;
}

// ---------------------------------------------------------------------------
// uploads / downloads
// ---------------------------------------------------------------------------
static void h2d(void *d, const void *h, size_t bytes, cudaStream_t st) {
  GWGB_REQUIRE(h != nullptr || bytes == 0, GWGB_E_INVALID, "NULL host pointer");
  GWGB_CUDA(cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, st));
}
static void d2h(void *h, const void *d, size_t bytes, cudaStream_t st) {
  GWGB_REQUIRE(h != nullptr || bytes == 0, GWGB_E_INVALID, "NULL host pointer");
  GWGB_CUDA(cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, st));
}

void Engine::upload_V(const double *V, int64_t n) {
  GWGB_REQUIRE(n == l_.flat_V, GWGB_E_INVALID,
               "V size " + std::to_string(n) + " does not match the layout (" + std::to_string(l_.flat_V) + ")");
  h2d(V_.p, V, (size_t)n * sizeof(double2), st_);
  GWGB_CUDA(cudaStreamSynchronize(st_));
  have_V_ = true;
  vt_ready_ = vcat_ready_ = oz_ready_ = false;  // rebuilt before the next solve
}

void Engine::set_reps(const double *orep, int64_t no, const double *auxrep, int64_t na) {
  GWGB_REQUIRE(no == l_.flat_orep && na == l_.flat_auxrep, GWGB_E_INVALID, "rotation matrix sizes do not match the layout");
  h2d(orep_.p, orep, (size_t)no * sizeof(double2), st_);
  h2d(auxrep_.p, auxrep, (size_t)na * sizeof(double2), st_);
  GWGB_CUDA(cudaStreamSynchronize(st_));
  have_reps_ = true;
  vt_ready_ = vcat_ready_ = oz_ready_ = false;  // rebuilt before the next solve
}

void Engine::set_transforms(const double *Tnt, const double *Ttn, const double *TntBF, const double *TtnFB,
                            const int64_t *ws, const double *tf, const double *tl) {
  GWGB_REQUIRE(Tnt && Ttn && TntBF && TtnFB && ws, GWGB_E_INVALID, "transform matrices must not be NULL");
  drop_graphs();  // the buffers below are reallocated
  Tnt_.alloc((size_t)nw_ * ncheb_);
  Ttn_.alloc((size_t)nts_ * nw_);
  TntBF_.alloc((size_t)nw_b_ * ncheb_);
  TtnFB_.alloc((size_t)nts_ * nw_b_);
  ws_.alloc(nw_);
  h2d(Tnt_.p, Tnt, Tnt_.n * sizeof(double2), st_);
  h2d(Ttn_.p, Ttn, Ttn_.n * sizeof(double2), st_);
  h2d(TntBF_.p, TntBF, TntBF_.n * sizeof(double2), st_);
  h2d(TtnFB_.p, TtnFB, TtnFB_.n * sizeof(double2), st_);
  h2d(ws_.p, ws, nw_ * sizeof(int64_t), st_);
  has_tct_ = tf && tl;
  if (has_tct_) {
    tct_f_.alloc(ncheb_);
    tct_l_.alloc(ncheb_);
    h2d(tct_f_.p, tf, ncheb_ * sizeof(double), st_);
    h2d(tct_l_.p, tl, ncheb_ * sizeof(double), st_);
  }
  GWGB_CUDA(cudaStreamSynchronize(st_));
  have_T_ = true;
}

void Engine::set_fock(const double *F, const double *S) {
  h2d(F_.p, F, F_.n * sizeof(double2), st_);
  h2d(S_.p, S, S_.n * sizeof(double2), st_);
  GWGB_CUDA(cudaStreamSynchronize(st_));
  have_F_ = true;
}

void Engine::set_G(const double *G) {
  h2d(Gall_.p, G, (size_t)nts_ * ns_ * l_.flat_ao * sizeof(double2), st_);
  GWGB_CUDA(cudaStreamSynchronize(st_));
}
void Engine::get_G(double *G) {
  d2h(G, Gall_.p, (size_t)nts_ * ns_ * l_.flat_ao * sizeof(double2), st_);
  GWGB_CUDA(cudaStreamSynchronize(st_));
}
void Engine::set_sigma(const double *S) {
  h2d(Sig_.p, S, Sig_.n * sizeof(double2), st_);
  GWGB_CUDA(cudaStreamSynchronize(st_));
}
void Engine::get_sigma(double *S) {
  d2h(S, Sig_.p, Sig_.n * sizeof(double2), st_);
  GWGB_CUDA(cudaStreamSynchronize(st_));
}
void Engine::set_P0(const double *P) {
  h2d(Pall_.p, P, (size_t)nts_ * l_.flat_aux * sizeof(double2), st_);
  GWGB_CUDA(cudaStreamSynchronize(st_));
}
void Engine::get_P0(double *P) {
  d2h(P, Pall_.p, (size_t)nts_ * l_.flat_aux * sizeof(double2), st_);
  GWGB_CUDA(cudaStreamSynchronize(st_));
}

// ---------------------------------------------------------------------------
// stages
// ---------------------------------------------------------------------------
void Engine::k_rotate_G() {
  launch_rotate(rotG_.p, (int)rotG_.n, nts_ * ns_, rot_smem_, Gall_.p, orep_.p, Gall_.p, st_);
}

void Engine::k_p0(int mirror) {
  const double pref = -1.0 / l_.nk * (ns_ == 1 ? 2.0 : 1.0);  // cugw_qkpt_block.cu:210, cugw_solver_block.cpp:303
  if (prec_ == GWGB_PREC_OZAKI) {  // sliced contractions: Z1 -> Z -> P0 per tau chunk
    GWGB_REQUIRE(oz_ready_, GWGB_E_STATE, "sliced-precision operands not prepared");
    launch_to_ffc(Gall_.p, Gff_.p, (int64_t)Gall_.n, st_);
    GWGB_CUDA(cudaMemsetAsync(Pall_.p, 0, Pall_.n * sizeof(double2), st_));  // blocks without contributions
    oz_run(oz_p0_, 0);
    lt_ran_p0_ = lt_on_;
    if (mirror) launch_mirror(Pall_.p, qoff_irr_.p, qsz_irr_.p, l_.ink, nts_, st_);
  } else if (prec_ != GWGB_PREC_FP64) {  // tcgen05 split contractions
    GWGB_REQUIRE((Zbuf_.p || !zbuf_elems_) && vcat_ready_, GWGB_E_STATE, "mixed-precision operands not prepared");
    for (const P0Chunk &ch : p0_chunks_)  // each chunk's slices are summed before the next chunk
      launch_p0_tc(prec_ == GWGB_PREC_BF16X3, pz_tasks_.p, (int)pz_tasks_.n, pz_smem_, pk_tiles_.p + ch.k0, ch.nk,
                   pr_tiles_.p + ch.r0, ch.nr, V_.p, Gall_.p, Zbuf_.p, Vcat_.p, Ppart_.p, Pall_.p, ns_, nts_,
                   ch.t0, ch.t1, pref, mirror, bad_.p + 2, st_);
  } else {
    launch_p0_fp64(p0_tiles_.p, (int)p0_tiles_.n, p0_maxo_, p0_contribs_.p, V_.p, Gall_.p, Part_.p, ns_, nts_,
                   fp64_smem_, st_);
    launch_reduce_slices(p0_red_.p, (int)p0_red_.n, Part_.p, Pall_.p, nts_, pref, mirror, st_);
  }
}

void Engine::k_pq(bool mirror_first) {
  if (mirror_first) launch_mirror(Pall_.p, qoff_irr_.p, qsz_irr_.p, l_.ink, nts_, st_);
  record(8);
  launch_transform(slab_p_fwd_.p, (int)slab_p_fwd_.n, max_cols_p_, TntBF_.p, nw_b_, ncheb_, 1, Pall_.p, Pw_.p, st_);
  record(9);
  launch_inverse(inv_w_.p, (int)inv_w_.n, l_.max_aux, Pw_.p, nullptr, nullptr, nullptr, beta_, 0.0, 0, bad_.p, st_);
  record(10);
  launch_transform(slab_p_bwd_.p, (int)slab_p_bwd_.n, max_cols_p_, TtnFB_.p, nts_, nw_b_, 0, Pw_.p, Pall_.p, st_);
  record(11);
}


void Engine::k_sigma() {
  if (prec_ == GWGB_PREC_OZAKI) {  // sliced contractions: W -> U -> Sigma per tau chunk
    GWGB_REQUIRE(oz_ready_, GWGB_E_STATE, "sliced-precision operands not prepared");
    launch_to_ffc(Gall_.p, Gff_.p, (int64_t)Gall_.n, st_);
    launch_to_ffc(Pall_.p, Pff_.p, (int64_t)Pall_.n, st_);
    GWGB_CUDA(cudaMemsetAsync(Sig_.p, 0, Sig_.n * sizeof(double2), st_));  // blocks without contributions
    oz_run(oz_sig_, lt_n_p0_);
    lt_ran_sig_ = lt_on_;
  } else if (prec_ != GWGB_PREC_FP64) {  // tcgen05 split contractions
    GWGB_REQUIRE(Wbuf_.p || !wbuf_elems_, GWGB_E_STATE, "mixed-precision work buffer missing");
    for (const SigChunk &ch : sig_chunks_) {
      launch_sigma_tc(prec_ == GWGB_PREC_BF16X3, sw_tiles_.p + ch.w0, ch.nw, sw_smem_, Bcat_.p,
                      sig_tiles1_.p + ch.uv0, ch.nuvt, uvt_smem_, sig_tiles1_.p + ch.uv0 + ch.nuvt, ch.nuv - ch.nuvt,
                      sig_contribs_.p, sig_wref_.p, Vt_.p, Gall_.p, Pall_.p, Wbuf_.p, Part_.p, ns_, uv_smem_,
                      ch.nuv_blocked, uv_smem_small_, ch.t0, bad_.p + 2, st_);
      launch_reduce_slices(uv_red_.p + ch.red0, ch.nred, Part_.p, Sig_.p, nts_, -1.0 / l_.nk, 0, st_);
    }
  } else {
    launch_sigma_fp64(sig_tiles_.p, (int)sig_tiles_.n, sig_maxo_, sig_contribs_.p, Vt_.p, Gall_.p, Pall_.p, Part_.p,
                      ns_, fp64_smem_, st_);
    launch_reduce_slices(sig_red_.p, (int)sig_red_.n, Part_.p, Sig_.p, nts_, -1.0 / l_.nk, 0, st_);
  }
}

void Engine::k_dyson() {
  launch_transform(slab_s_fwd_.p, (int)slab_s_fwd_.n, max_cols_g_, Tnt_.p, nw_, ncheb_, 1, Sig_.p, Ww_.p, st_);
  launch_inverse(inv_d_.p, (int)inv_d_.n, l_.max_ao, Ww_.p, S_.p, F_.p, ws_.p, beta_, 0.0, 1, bad_.p + 1, st_);
  launch_transform(slab_g_bwd_.p, (int)slab_g_bwd_.n, max_cols_g_, Ttn_.p, nts_, nw_, 0, Ww_.p, Gall_.p, st_);
  if (has_tct_) {
    GWGB_CUDA(cudaMemsetAsync(leak_.p, 0, 2 * sizeof(unsigned long long), st_));
    launch_leakage(slab_g_bwd_.p, (int)slab_g_bwd_.n, Gall_.p, tct_f_.p, tct_l_.p, ncheb_, leak_.p, st_);
  }
}

void Engine::check_device_flags() {
  int bad[4] = {0, 0, 0, 0};
  GWGB_CUDA(cudaMemcpy(bad, bad_.p, sizeof(bad), cudaMemcpyDeviceToHost));
  if (bad[0] || bad[1] || bad[2]) {
    GWGB_CUDA(cudaMemset(bad_.p, 0, sizeof(bad)));
    if (bad[2]) throw Error(GWGB_E_TIMEOUT, "a tensor-core MMA completion wait ran out (tcgen05 commit not observed)");
    throw Error(GWGB_E_NUMERIC, bad[0] ? "singular block in the W~ solve (1 - P~0)" : "singular block in Dyson");
  }
}

void Engine::finish_stats(bool with_dyson, bool with_gw, bool with_pq, bool with_dy) {
  GWGB_CUDA(cudaStreamSynchronize(st_));
  check_device_flags();
  gwgb_stats s{};
  if (with_gw) {
    s.rotate_G_ms = elapsed(0, 1);
    s.p0_ms = elapsed(1, 2);
    s.pq_ms = elapsed(2, 3);
    s.rotate_P_ms = elapsed(3, 4);
    s.sigma_ms = elapsed(4, 5);
    s.p0_flops = p0_flops_;
    s.sigma_flops = sig_flops_;
  }
  if (with_dyson) {
    s.dyson_ms = elapsed(5, 6);
    if (has_tct_) {
      unsigned long long lk[2];
      GWGB_CUDA(cudaMemcpy(lk, leak_.p, sizeof(lk), cudaMemcpyDeviceToHost));
      double f, la;
      std::memcpy(&f, &lk[0], 8);
      std::memcpy(&la, &lk[1], 8);
      s.leakage = f > 0 ? la / f : 0.0;
    }
  }
  s.total_ms = elapsed(with_gw ? 0 : 5, with_dyson ? 6 : 5);
  if (with_pq) {
    s.transform_ms += elapsed(8, 9) + elapsed(10, 11);
    s.transform_bytes += tr_bytes_pq_;
    s.transform_flops += tr_flops_pq_;
    s.solve_ms += elapsed(9, 10);
    s.solve_flops += solve_flops_pq_;
  }
  if (with_dy) {
    s.transform_ms += elapsed(5, 12) + elapsed(13, 14);
    s.transform_bytes += tr_bytes_dy_;
    s.transform_flops += tr_flops_dy_;
    s.solve_ms += elapsed(12, 13);
    s.solve_flops += solve_flops_dy_;
  }
  int64_t launches = 0;
  if (with_gw) {
    const bool tc = tc_split();
    int64_t sgt = 0, p0t = 0;
    for (const SigChunk &ch : sig_chunks_)
      sgt += (ch.nw ? 1 : 0) + (ch.nuvt ? 1 : 0) + (ch.nuv_blocked ? 1 : 0) +
             (ch.nuv - ch.nuvt > ch.nuv_blocked ? 1 : 0) + (ch.nred ? 1 : 0);
    for (const P0Chunk &ch : p0_chunks_) p0t += (pz_tasks_.n ? 1 : 0) + (ch.nk ? 1 : 0) + (ch.nr ? 1 : 0);
    const int64_t p0 = tc ? p0t
                          : (p0_tiles_.n ? 1 : 0) + (p0_red_.n ? 1 : 0);
    const int64_t sg = tc ? sgt
                          : (sig_tiles_.n ? 1 : 0) + (sig_red_.n ? 1 : 0);
    if (prec_ == GWGB_PREC_OZAKI) {
      int64_t a = 1, b = 2;  // G (and P~) to float-float
      for (const OzLaunch &x : oz_p0_) a += x.n ? 1 : 0;
      for (const OzLaunch &x : oz_sig_) b += x.n ? 1 : 0;
      launches += (rotG_.n ? 1 : 0) + a + 1 + 3 + b;
    } else
    launches += (rotG_.n ? 1 : 0) + p0 + 3 + sg;
  }
  if (with_dyson) launches += 3 + (has_tct_ ? 1 : 0);
  s.kernel_launches = launches;
  stats_ = s;
}

void Engine::solve_P0() {
  require_ready(false);
  prepare_operands();
  record(0);
  k_rotate_G();
  record(1);
  k_p0(0);
  launch_zero_upper(Pall_.p, qoff_irr_.p, qsz_irr_.p, l_.ink, nts_, st_);
  for (int i = 2; i <= 6; ++i) record(i);
  finish_stats(false, true);
}

void Engine::solve_Pq() {
  require_ready(true);
  record(0); record(1); record(2);
  k_pq(true);
  for (int i = 3; i <= 6; ++i) record(i);
  finish_stats(false, true, true);
}

void Engine::solve_sigma() {
  require_ready(false);
  prepare_operands();
  record(0);
  k_rotate_G();
  record(1);
  k_p0(1);
  record(2);
  record(3);
  record(4);
  k_sigma();
  record(5);
  record(6);
  finish_stats(false, true);
}

// Hartree term of HF from the handle's G at tau = 0 (a density matrix): J over
// the stored k, [flat_ao].  Closed-shell factor 2 for ns = 1.
void Engine::hf_hartree(double *J) {
  GWGB_REQUIRE(J, GWGB_E_INVALID, "NULL J");
  require_ready(false);
  k_rotate_G();
  launch_hartree(hart_ct_.p, (int)hart_ct_.n, hart_ci_.p, hart_jt_.p, (int)hart_jt_.n, hart_ji_.p, V_.p, Gall_.p,
                 ns_, (ns_ == 1 ? 2.0 : 1.0) / l_.nk, hart_c_.p, hart_J_.p, st_);
  GWGB_CUDA(cudaMemcpyAsync(J, hart_J_.p, (size_t)l_.flat_ao * sizeof(double2), cudaMemcpyDeviceToHost, st_));
  GWGB_CUDA(cudaStreamSynchronize(st_));
  check_device_flags();
}

// The Sigma stage alone on the handle's G and P buffers (P0 is not recomputed).
void Engine::solve_sigma_from_P() {
  require_ready(false);
  prepare_operands();
  record(0);
  k_rotate_G();
  for (int i = 1; i <= 4; ++i) record(i);
  k_sigma();
  record(5);
  record(6);
  finish_stats(false, true);
}

void Engine::solve() {
  require_ready(true);
  prepare_operands();
  record(0);
  k_rotate_G();
  record(1);
  k_p0(1);
  record(2);
  k_pq(false);
  record(3);
  record(4);
  k_sigma();
  record(5);
  record(6);
  finish_stats(false, true, true);
}

void Engine::dyson(double mu) {
  GWGB_REQUIRE(have_T_, GWGB_E_STATE, "transform matrices have not been set");
  GWGB_REQUIRE(have_F_, GWGB_E_STATE, "F and S have not been set");
  // mu enters the inverse kernel by value here (no graph)
  record(5);
  launch_transform(slab_s_fwd_.p, (int)slab_s_fwd_.n, max_cols_g_, Tnt_.p, nw_, ncheb_, 1, Sig_.p, Ww_.p, st_);
  record(12);
  launch_inverse(inv_d_.p, (int)inv_d_.n, l_.max_ao, Ww_.p, S_.p, F_.p, ws_.p, beta_, mu, 1, bad_.p + 1, st_);
  record(13);
  launch_transform(slab_g_bwd_.p, (int)slab_g_bwd_.n, max_cols_g_, Ttn_.p, nts_, nw_, 0, Ww_.p, Gall_.p, st_);
  record(14);
  if (has_tct_) {
    GWGB_CUDA(cudaMemsetAsync(leak_.p, 0, 2 * sizeof(unsigned long long), st_));
    launch_leakage(slab_g_bwd_.p, (int)slab_g_bwd_.n, Gall_.p, tct_f_.p, tct_l_.p, ncheb_, leak_.p, st_);
  }
  record(6);
  finish_stats(true, false, false, true);
}

void Engine::iteration(double mu) {
  require_ready(true);
  prepare_operands();
  GWGB_REQUIRE(have_F_, GWGB_E_STATE, "F and S have not been set");
  // The graph holds mu by value; rebuild when it changes.
  if (!graph_exec_ || *mu_host_ != mu) {
    if (graph_exec_) {
      cudaGraphExecDestroy(graph_exec_);
      graph_exec_ = nullptr;
    }
    *mu_host_ = mu;
    cudaGraph_t g;
    GWGB_CUDA(cudaStreamBeginCapture(st_, cudaStreamCaptureModeThreadLocal));
    capturing_ = true;
    try {
    record(0);
    k_rotate_G();
    record(1);
    k_p0(1);
    record(2);
    k_pq(false);
    record(3);
    record(4);
    k_sigma();
    record(5);
    launch_transform(slab_s_fwd_.p, (int)slab_s_fwd_.n, max_cols_g_, Tnt_.p, nw_, ncheb_, 1, Sig_.p, Ww_.p, st_);
    record(12);
    launch_inverse(inv_d_.p, (int)inv_d_.n, l_.max_ao, Ww_.p, S_.p, F_.p, ws_.p, beta_, mu, 1, bad_.p + 1, st_);
    record(13);
    launch_transform(slab_g_bwd_.p, (int)slab_g_bwd_.n, max_cols_g_, Ttn_.p, nts_, nw_, 0, Ww_.p, Gall_.p, st_);
    record(14);
    if (has_tct_) {
      GWGB_CUDA(cudaMemsetAsync(leak_.p, 0, 2 * sizeof(unsigned long long), st_));
      launch_leakage(slab_g_bwd_.p, (int)slab_g_bwd_.n, Gall_.p, tct_f_.p, tct_l_.p, ncheb_, leak_.p, st_);
    }
    record(6);
    } catch (...) {
      capturing_ = false;
      cudaGraph_t dead = nullptr;
      cudaStreamEndCapture(st_, &dead);
      if (dead) cudaGraphDestroy(dead);
      throw;
    }
    capturing_ = false;
    cudaError_t e = cudaStreamEndCapture(st_, &g);
    GWGB_CUDA(e);
    GWGB_CUDA(cudaGraphInstantiate(&graph_exec_, g, 0));
    cudaGraphDestroy(g);
  }
  GWGB_CUDA(cudaGraphLaunch(graph_exec_, st_));
  finish_stats(true, true, true, true);
}


// ---------------------------------------------------------------------------
// self-consistent loop (no counterpart in the reference; formulas in gwgb.h)
// ---------------------------------------------------------------------------
void Engine::set_hcore(const double *H) {
  GWGB_REQUIRE(H, GWGB_E_INVALID, "NULL H");
  if (!Hc_.p) Hc_.alloc((size_t)ns_ * l_.flat_ao);
  h2d(Hc_.p, H, Hc_.n * sizeof(double2), st_);
  GWGB_CUDA(cudaStreamSynchronize(st_));
  if (!have_H_) drop_graphs();
  have_H_ = true;
}

void Engine::set_energy_matrix(const double *M, int n) {
  GWGB_REQUIRE(M, GWGB_E_INVALID, "NULL energy matrix");
  GWGB_REQUIRE(n == ncheb_, GWGB_E_INVALID, "energy matrix must be (nts-2) x (nts-2)");
  std::vector<double2> m((size_t)n * n);
  for (size_t i = 0; i < m.size(); ++i) m[i] = make_double2(M[i], 0.0);
  if (!Me_.p) Me_.alloc(m.size());
  h2d(Me_.p, m.data(), m.size() * sizeof(double2), st_);
  GWGB_CUDA(cudaStreamSynchronize(st_));
  if (!have_M_) drop_graphs();
  have_M_ = true;
}

void Engine::check_mu_search(const gwgb_mu_search &ms) const {
  GWGB_REQUIRE(ms.max_evals >= 2 && ms.max_evals <= 64, GWGB_E_INVALID, "max_evals must be in [2, 64]");
  GWGB_REQUIRE(ms.step > 0.0 && std::isfinite(ms.step), GWGB_E_INVALID, "mu search step must be positive");
  GWGB_REQUIRE(ms.tol > 0.0 && std::isfinite(ms.tol), GWGB_E_INVALID, "mu search tolerance must be positive");
  GWGB_REQUIRE(std::isfinite(ms.mu0) && std::isfinite(ms.n_electrons), GWGB_E_INVALID, "mu0 and N must be finite");
}

void Engine::init_mu_state(const gwgb_mu_search &ms) {
  MuState h{};
  h.target = ms.n_electrons;
  h.tol = ms.tol;
  h.mu = h.best_mu = ms.mu0;
  h.best_f = 1e300;
  h2d(mus_.p, &h, sizeof(MuState), st_);
  GWGB_CUDA(cudaMemsetAsync(counter_.p, 0, sizeof(int), st_));
  GWGB_CUDA(cudaStreamSynchronize(st_));
}

// Ww_ holds Sigma(i w).  Ends with *mu_dev_ = the best mu found.
void Engine::k_mu_search(const gwgb_mu_search &ms) {
  const double nscale = -(2.0 / ns_) / l_.nk;
  const int *done = reinterpret_cast<const int *>(reinterpret_cast<const char *>(mus_.p) + offsetof(MuState, done));
  launch_mu_begin(mus_.p, mu_dev_.p, ms.step, st_);
  for (int e = 0; e < ms.max_evals; ++e) {
    launch_inverse(inv_d_.p, (int)inv_d_.n, l_.max_ao, Ww_.p, S_.p, F_.p, ws_.p, beta_, 0.0, 1, bad_.p + 1, st_,
                   mu_dev_.p, Wg_.p, done);
    // G(beta) only: the last row of Ttn
    launch_transform(slab_g_bwd_.p, (int)slab_g_bwd_.n, max_cols_g_, Ttn_.p + (int64_t)(nts_ - 1) * nw_, 1, nw_, 0,
                     Wg_.p, Gb_.p, st_);
    launch_mu_update(tr_tasks_.p, (int)tr_tasks_.n, Gb_.p, S_.p, nscale, mus_.p, mu_dev_.p,
                     e == ms.max_evals - 1, st_);
  }
}

void Engine::k_dyson_dev() {
  launch_inverse(inv_d_.p, (int)inv_d_.n, l_.max_ao, Ww_.p, S_.p, F_.p, ws_.p, beta_, 0.0, 1, bad_.p + 1, st_,
                 mu_dev_.p);
  launch_transform(slab_g_bwd_.p, (int)slab_g_bwd_.n, max_cols_g_, Ttn_.p, nts_, nw_, 0, Ww_.p, Gall_.p, st_);
  if (has_tct_) {
    GWGB_CUDA(cudaMemsetAsync(leak_.p, 0, 2 * sizeof(unsigned long long), st_));
    launch_leakage(slab_g_bwd_.p, (int)slab_g_bwd_.n, Gall_.p, tct_f_.p, tct_l_.p, ncheb_, leak_.p, st_);
  }
}

void Engine::k_energy_record(bool with_energy) {
  if (with_energy)
    launch_transform(slab_e_.p, (int)slab_e_.n, max_cols_g_, Me_.p, ncheb_, ncheb_, 1, Gall_.p, Hm_.p, st_);
  EnergyArgs a{};
  a.tasks = tr_tasks_.p;
  a.ntasks = (int)tr_tasks_.n;
  a.ncheb = ncheb_;
  a.nts = nts_;
  a.ldt = (int64_t)ns_ * l_.flat_ao;
  a.sig = Sig_.p;
  a.hm = Hm_.p;
  a.g = Gall_.p;
  a.f = F_.p;
  a.hc = have_H_ ? Hc_.p : nullptr;
  a.s = S_.p;
  a.st = mus_.p;
  a.leak = has_tct_ ? leak_.p : nullptr;
  a.nscale = -(2.0 / ns_) / l_.nk;
  a.ecorr_scale = -(1.0 / ns_) / l_.nk;
  a.eone_scale = -(1.0 / ns_) / l_.nk;
  a.precision = prec_;
  a.with_energy = with_energy ? 1 : 0;
  a.rec = recs_.p;
  a.counter = counter_.p;
  launch_energy_record(a, st_);
}

void Engine::k_sc_iteration(double alpha, const gwgb_mu_search &ms) {
  k_rotate_G();
  k_p0(1);
  k_pq(false);
  k_sigma();
  launch_mix(Sig_.p, Sold_.p, (int64_t)Sig_.n, alpha, st_);
  launch_transform(slab_s_fwd_.p, (int)slab_s_fwd_.n, max_cols_g_, Tnt_.p, nw_, ncheb_, 1, Sig_.p, Ww_.p, st_);
  k_mu_search(ms);
  k_dyson_dev();
  k_energy_record(have_M_);
}

template <typename F>
void Engine::capture(cudaGraphExec_t *exec, F &&body) {
  cudaGraph_t g = nullptr;
  GWGB_CUDA(cudaStreamBeginCapture(st_, cudaStreamCaptureModeThreadLocal));
  capturing_ = true;
  try {
    body();
  } catch (...) {
    capturing_ = false;
    cudaGraph_t dead = nullptr;
    cudaStreamEndCapture(st_, &dead);
    if (dead) cudaGraphDestroy(dead);
    throw;
  }
  capturing_ = false;
  GWGB_CUDA(cudaStreamEndCapture(st_, &g));
  const cudaError_t e = cudaGraphInstantiate(exec, g, 0);
  cudaGraphDestroy(g);
  GWGB_CUDA(e);
}

gwgb_sc_record Engine::read_record(int i) {
  gwgb_sc_record r{};
  GWGB_CUDA(cudaMemcpy(&r, recs_.p + i, sizeof(r), cudaMemcpyDeviceToHost));
  return r;
}

void Engine::find_mu(const gwgb_mu_search &ms, double *mu_out, double *n_out) {
  GWGB_REQUIRE(have_T_, GWGB_E_STATE, "transform matrices have not been set");
  GWGB_REQUIRE(have_F_, GWGB_E_STATE, "F and S have not been set");
  check_mu_search(ms);
  init_mu_state(ms);
  record(5);
  launch_transform(slab_s_fwd_.p, (int)slab_s_fwd_.n, max_cols_g_, Tnt_.p, nw_, ncheb_, 1, Sig_.p, Ww_.p, st_);
  k_mu_search(ms);
  k_dyson_dev();
  k_energy_record(false);
  record(6);
  finish_stats(true, false);
  const gwgb_sc_record r = read_record(0);
  if (mu_out) *mu_out = r.mu;
  if (n_out) *n_out = r.n_electrons;
}

void Engine::energy(double *e_corr, double *e_one) {
  GWGB_REQUIRE(!e_corr || have_M_, GWGB_E_STATE, "the energy matrix has not been set");
  GWGB_REQUIRE(!e_one || have_H_, GWGB_E_STATE, "the core Hamiltonian has not been set");
  GWGB_REQUIRE(have_F_, GWGB_E_STATE, "F and S have not been set");
  GWGB_CUDA(cudaMemsetAsync(counter_.p, 0, sizeof(int), st_));
  k_energy_record(have_M_);
  GWGB_CUDA(cudaStreamSynchronize(st_));
  check_device_flags();
  const gwgb_sc_record r = read_record(0);
  if (e_corr) *e_corr = r.e_corr;
  if (e_one) *e_one = r.e_one;
}

void Engine::sc_loop(int niter, double alpha, const gwgb_mu_search &ms, int final_fp64, gwgb_sc_record *out) {
  require_ready(true);
  GWGB_REQUIRE(have_F_, GWGB_E_STATE, "F and S have not been set");
  GWGB_REQUIRE(out, GWGB_E_INVALID, "NULL record array");
  GWGB_REQUIRE(niter >= 1 && niter <= 100000, GWGB_E_INVALID, "niter must be in [1, 100000]");
  GWGB_REQUIRE(alpha > 0.0 && alpha <= 1.0, GWGB_E_INVALID, "mixing alpha must be in (0, 1]");
  check_mu_search(ms);
  prepare_operands();
  if ((int)recs_.n < niter) {  // the graph records through recs_.p
    drop_graphs();
    recs_.alloc((size_t)niter);
  }
  init_mu_state(ms);
  GWGB_CUDA(cudaMemcpyAsync(Sold_.p, Sig_.p, Sig_.n * sizeof(double2), cudaMemcpyDeviceToDevice, st_));
  const bool same = sc_exec_ && alpha == sc_alpha_ && std::memcmp(&ms, &sc_ms_, sizeof(ms)) == 0;
  if (!same && sc_exec_) {
    cudaGraphExecDestroy(sc_exec_);
    sc_exec_ = nullptr;
  }
  const int prec0 = prec_;
  const int nmain = (final_fp64 && prec0 != GWGB_PREC_FP64) ? niter - 1 : niter;
  GWGB_CUDA(cudaEventRecord(sc_ev_[0], st_));
  if (nmain > 0) {
    if (!sc_exec_) {
      capture(&sc_exec_, [&] { k_sc_iteration(alpha, ms); });
      sc_alpha_ = alpha;
      sc_ms_ = ms;
    }
    for (int i = 0; i < nmain; ++i) GWGB_CUDA(cudaGraphLaunch(sc_exec_, st_));
  }
  if (nmain < niter) {  // the last iteration with the FP64 contractions
    GWGB_CUDA(cudaStreamSynchronize(st_));
    set_precision(GWGB_PREC_FP64);
    capture(&sc_exec_, [&] { k_sc_iteration(alpha, ms); });
    sc_alpha_ = alpha;
    sc_ms_ = ms;
    GWGB_CUDA(cudaGraphLaunch(sc_exec_, st_));
    GWGB_CUDA(cudaStreamSynchronize(st_));
    set_precision(prec0);
  }
  GWGB_CUDA(cudaEventRecord(sc_ev_[1], st_));
  GWGB_CUDA(cudaStreamSynchronize(st_));
  check_device_flags();
  GWGB_CUDA(cudaMemcpy(out, recs_.p, (size_t)niter * sizeof(gwgb_sc_record), cudaMemcpyDeviceToHost));
  float ms_total = 0;
  GWGB_CUDA(cudaEventElapsedTime(&ms_total, sc_ev_[0], sc_ev_[1]));
  gwgb_stats st{};
  st.total_ms = ms_total / niter;
  st.p0_flops = p0_flops_;
  st.sigma_flops = sig_flops_;
  st.leakage = out[niter - 1].leakage;
  stats_ = st;
}

}  // namespace gwgb

#include "refproxy.cuh"

// ===========================================================================
// C ABI
// ===========================================================================
using gwgb::Engine;

struct gwgb_handle_s {
  Engine *e;
};

template <typename F>
static int guarded(F &&f) {
  try {
    f();
    return GWGB_OK;
  } catch (const gwgb::Error &e) {
    gwgb::g_last_error = e.what();
    return e.code;
  } catch (const std::bad_alloc &) {
    gwgb::g_last_error = "host allocation failed";
    return GWGB_E_NOMEM;
  } catch (const std::exception &e) {
    gwgb::g_last_error = e.what();
    return GWGB_E_INVALID;
  }
}

template <typename F>
static int on_handle(gwgb_handle h, F &&f) {
  if (!h || !h->e) {
    gwgb::g_last_error = "NULL handle";
    return GWGB_E_INVALID;
  }
  std::lock_guard<std::mutex> lk(h->e->mu_lock);
  return guarded([&] {
    GWGB_CUDA(cudaSetDevice(h->e->device()));
    f(*h->e);
  });
}

extern "C" {

const char *gwgb_version(void) {
  return "gwgb 0.5 (sm_103a; FP64, sliced BF16 (Ozaki), TF32x3 and BF16x3 contraction paths)";
}

const char *gwgb_last_error(void) { return gwgb::g_last_error.c_str(); }

int gwgb_create(const gwgb_params *params, const gwgb_layout *layout, gwgb_handle *out) {
  return guarded([&] {
    GWGB_REQUIRE(params && layout && out, GWGB_E_INVALID, "NULL argument to gwgb_create");
    *out = nullptr;
    auto *h = new gwgb_handle_s{nullptr};
    try {
      h->e = new Engine(*params, *layout);
    } catch (...) {
      delete h;
      throw;
    }
    *out = h;
  });
}

int gwgb_destroy(gwgb_handle h) {
  if (!h) return GWGB_OK;
  int rc = guarded([&] { delete h->e; });
  delete h;
  return rc;
}

#define GWGB_FORWARD(name, sig_args, call)                                       \
  int name sig_args { return on_handle(h, [&](Engine &e) { call; }); }

GWGB_FORWARD(gwgb_set_precision, (gwgb_handle h, int32_t precision), e.set_precision(precision))
GWGB_FORWARD(gwgb_upload_V, (gwgb_handle h, const double *V, int64_t n), e.upload_V(V, n))
GWGB_FORWARD(gwgb_set_reps, (gwgb_handle h, const double *o, int64_t no, const double *a, int64_t na),
             e.set_reps(o, no, a, na))
GWGB_FORWARD(gwgb_set_transforms,
             (gwgb_handle h, const double *Tnt, const double *Ttn, const double *TntBF, const double *TtnFB,
              const int64_t *ws, const double *tf, const double *tl),
             e.set_transforms(Tnt, Ttn, TntBF, TtnFB, ws, tf, tl))
GWGB_FORWARD(gwgb_set_fock, (gwgb_handle h, const double *F, const double *S), e.set_fock(F, S))
GWGB_FORWARD(gwgb_set_G, (gwgb_handle h, const double *G), e.set_G(G))
GWGB_FORWARD(gwgb_get_G, (gwgb_handle h, double *G), e.get_G(G))
GWGB_FORWARD(gwgb_set_sigma, (gwgb_handle h, const double *S), e.set_sigma(S))
GWGB_FORWARD(gwgb_get_sigma, (gwgb_handle h, double *S), e.get_sigma(S))
GWGB_FORWARD(gwgb_set_P0, (gwgb_handle h, const double *P), e.set_P0(P))
GWGB_FORWARD(gwgb_get_P0, (gwgb_handle h, double *P), e.get_P0(P))
GWGB_FORWARD(gwgb_solve_P0, (gwgb_handle h), e.solve_P0())
GWGB_FORWARD(gwgb_solve_Pq, (gwgb_handle h), e.solve_Pq())
GWGB_FORWARD(gwgb_solve_sigma, (gwgb_handle h), e.solve_sigma())
GWGB_FORWARD(gwgb_solve_sigma_from_P, (gwgb_handle h), e.solve_sigma_from_P())
GWGB_FORWARD(gwgb_hf_hartree, (gwgb_handle h, double *J), e.hf_hartree(J))
GWGB_FORWARD(gwgb_solve, (gwgb_handle h), e.solve())
GWGB_FORWARD(gwgb_dyson, (gwgb_handle h, double mu), e.dyson(mu))
GWGB_FORWARD(gwgb_iteration, (gwgb_handle h, double mu), e.iteration(mu))
GWGB_FORWARD(gwgb_get_stats, (gwgb_handle h, gwgb_stats *out), GWGB_REQUIRE(out, GWGB_E_INVALID, "NULL stats"); e.stats(out))
GWGB_FORWARD(gwgb_synchronize, (gwgb_handle h), e.synchronize())
GWGB_FORWARD(gwgb_set_launch_timing, (gwgb_handle h, int32_t on), e.set_launch_timing(on))
GWGB_FORWARD(gwgb_get_launch_stats, (gwgb_handle h, gwgb_launch_stat *out, int32_t max, int32_t *n),
             e.launch_stats(out, max, n))
GWGB_FORWARD(gwgb_test_raise_status, (gwgb_handle h, int32_t which), e.test_raise_status(which))

int gwgb_test_wait_timeout(int32_t device, int32_t polls) {
  int status = 0;
  const int rc = guarded([&] {
    GWGB_REQUIRE(polls >= 1 && polls <= 10000000, GWGB_E_INVALID, "polls must be in [1, 1e7]");
    GWGB_CUDA(cudaSetDevice(device));
    status = gwgb::run_wait_timeout_test(polls);
  });
  if (rc != GWGB_OK) return rc;
  if (status) {
    gwgb::g_last_error = "a bounded device-side wait ran out (test hook)";
    return GWGB_E_TIMEOUT;
  }
  return GWGB_OK;
}

GWGB_FORWARD(gwgb_set_hcore, (gwgb_handle h, const double *H), e.set_hcore(H))
GWGB_FORWARD(gwgb_refproxy_run, (gwgb_handle h, int32_t nt_batch, int32_t nstreams, gwgb_proxy_stats *out),
             e.refproxy(nt_batch, nstreams, out))
GWGB_FORWARD(gwgb_refproxy_get, (gwgb_handle h, double *P0, double *Sigma), e.refproxy_get(P0, Sigma))
GWGB_FORWARD(gwgb_set_energy_matrix, (gwgb_handle h, const double *M, int32_t n), e.set_energy_matrix(M, n))
GWGB_FORWARD(gwgb_find_mu, (gwgb_handle h, const gwgb_mu_search *ms, double *mu_out, double *n_out),
             GWGB_REQUIRE(ms, GWGB_E_INVALID, "NULL mu search"); e.find_mu(*ms, mu_out, n_out))
GWGB_FORWARD(gwgb_energy, (gwgb_handle h, double *e_corr, double *e_one), e.energy(e_corr, e_one))
GWGB_FORWARD(gwgb_sc_loop,
             (gwgb_handle h, int32_t niter, double alpha, const gwgb_mu_search *ms, int32_t final_fp64,
              gwgb_sc_record *out),
             GWGB_REQUIRE(ms, GWGB_E_INVALID, "NULL mu search"); e.sc_loop(niter, alpha, *ms, final_fp64, out))

}  // extern "C"
