// capi.cu -- the C ABI of include/nemo_gpu.h: context life cycle, domain derivation,
// module-field binding, and the entry points that replace the bodies of NEMO's
// tra_adv_fct, tra_ldf_lap/iso, tra_zdf_imp, dyn_spg_ts, lbc_lnk and glob_sum.
//
// The host derives the masks, level indices and metric products from the domain
// description with the formulas of dommsk.F90, domzgr.F90, domhgr.F90 and
// domain.F90 in FP64, then uploads them once (rounded to FP32 for a mixed context).
// All later work is asynchronous on the context's stream.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <initializer_list>
#include <map>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "../../include/nemo_gpu.h"
#include "adj.h"
#include "step.h"
#include "triad.h"
#include "eos80.h"
#include "nemo_sin.h"
#include "launch.h"

using namespace nemo;

namespace {

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
};

// Per-precision device copy of the derived domain.
template <class T>
struct DomStore {
  Dom<T> d{};
  std::vector<void*> owned;
};

}  // namespace

struct nemo_ctx {
  int jpi = 0, jpj = 0, jpk = 0, nmem = 1, prec = NEMO_PREC_FP64;
  long n2 = 0, n3 = 0;
  nemo_namelist nam{};
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::string err;
  int nsm = 0;
  // derived host domain (FP64)
  std::vector<double> e1t, e2t, e1u, e2u, e1v, e2v, e1f, e2f, ff_f, ff_t;
  std::vector<double> r1_e1t, r1_e2t, r1_e1u, r1_e2u, r1_e1v, r1_e2v, e1e2t, r1_e1e2t, e1e2u, e1e2v;
  std::vector<double> r1_e1e2u, r1_e1e2v, e2_e1u, e1_e2v, r1_e1e2f;
  std::vector<double> ssmask, ssumask, ssvmask, tmask_i, ht_0, hu_0, hv_0, r1_hu_0, r1_hv_0;
  std::vector<double> zwz, ftne, ftnw, ftse, ftsw;
  std::vector<ColInfo> ci;
  std::vector<uint8_t> mbkt;
  std::vector<double> e3_0[5];  // t,u,v,w,f rest state (3-D)
  bool e3_uniform[5] = {false, false, false, false, false};
  // spg
  int nn_baro = 0, icycle = 0;
  int nksr = 0;  // tra_qsr: level of light extinction of the two bands
  int nlb10 = 0;  // zdf_mxl: the first W-level below 10 m
  double rdtbt = 0;
  std::vector<double> wgt1, wgt2;
  double* d_wgt1 = nullptr;
  double* d_wgt2 = nullptr;
  float* d_wgtf = nullptr;  // mixed form: wgt1 split as hi | lo, and wgt2, as floats
  std::vector<float> wgtf;
  int ring0 = 0;
  // device domain
  DomStore<double> dd;
  DomStore<float> df;
  // bound fields
  void* f[NEMO_F_COUNT] = {};
  // work arrays
  void* fct_w[6] = {};
  void* fct_ztw = nullptr;
  void* iso_w[3] = {};         // iso-neutral fluxes zftu, zftv, ztfw
  void* adj_w[4] = {};         // iso-neutral adjoint: G and the gradient adjoints
  double* spgadj_w = nullptr;  // dyn_spg_ts adjoint: 18 (jpi,jpj) arrays per member
  double* wzvadj_w = nullptr;  // wzv adjoint: one (jpi,jpj,jpk) array per member
  int adj_kjpt = 0;
  void* slp_w = nullptr;       // ldf_slp work: 4 3-D and 6 2-D arrays per member
  void* rab_w = nullptr;       // the model step's before expansion ratios rab_b (jpi,jpj,jpk,2)
  void* rab_n = nullptr;       // and the now ones rab_n, with the vertical physics
  void* zphy_w = nullptr;      // zdf_phy work: sh2, apdlr and the TKE system, 5 x n3 per member
  void* zdyn_w = nullptr;      // dyn_zdf work: the implicit viscosity system, 2 x n3 per member
  double* fadj_w = nullptr;    // FCT adjoint with kn_fct_v = 4: 2 x n3 per member
  double* usr_s = nullptr;     // usrdef_sbc: the step's scalars (7), written before each step
  double usr_zsurf = 0.0;      // usrdef_sbc: GLOB_SUM(tmask(:,:,1))
  void* blp_w = nullptr;       // tra_ldf_blp: the first laplacian (jpi,jpj,jpk,kjpt) per member
  int blp_kjpt = 0;
  int iso_kjpt = 0;
  int fct_kjpt = 0;
  void* spg_w[5] = {};
  void* spg_cor[5] = {};  // variable volume: Coriolis factors of each member
  void* ring[3] = {};
  void* spg_x[8] = {};  // fx (2 slots), fy (2 slots), du, dv, cu, cv, zmu, zmv
  float* spg_ff = nullptr;  // mixed form: compensated sub-step sums, 10 x nmem x n2
  unsigned int* bar_mem = nullptr;  // count, gen
  int* err_flag = nullptr;
  // EOS-80 tables (eos80.h): raw FP64 [3][4][7][7]; FP32 re-expanded about s0 =
  // sqrt((35 + 20) / 40), and the density at (35 psu, 0 degC, 0 m)
  double* e80_raw = nullptr;
  float* e80_tay = nullptr;
  double e80_s0 = 0.0, e80_rho0 = 0.0;
  // stp_ctl (block partials, per-member results, the blow-up flag) and dia_hsb
  double* ctl_part = nullptr;
  double* ctl_out = nullptr;
  unsigned long long* ctl_idx = nullptr;  // first indices of the extremes (4 per member)
  int* ctl_flag = nullptr;
  int ctl_nblk = 0;
  int hsb_nblk = 0;  // dia_hsb's block partials (2 per SM)
  int someoce = 0;  // the domain has ocean points (stpctl.F90:111)
  bool hsb_on = false;
  double* hsb_mem = nullptr;  // surf, tmask_h; ssh, ssh heat, ssh salt (x nmem); e3t, heat, salt (x nmem)
  double* hsb_part = nullptr;
  double* hsb_state = nullptr;  // 8 a member: frc_v, frc_t, frc_s, frc_wn_t, frc_wn_s, surf_tot
  double* hsb_out = nullptr;    // NEMO_HSB_N a member
  long long bar_spins = 4000000;
  int tma_polls = 1 << 16;  // bound of each wait of a TMA kernel on its tensor copies
  int bar_extra = 0;
  int p2_blocks = 0;
  int p2_cache = 0;  // the sub-step kernel keeps its constants in shared memory
  int p2_hot = 0;    // the sub-step kernel is k_spg_p2_ene (mixed, linear free surface, ENE/MIX)
  bool no_p2_hot = false;  // keep the general sub-step kernel (tests compare both)
  double* gs_part = nullptr;
  double* gs_out = nullptr;
  int gs_nblk = 0;
  double r2dt = 0;
  std::map<int, cudaGraphExec_t> graphs;
  bool graphs_ok = true;
  // per-routine timing of the hot path (the ln_timing of timing.F90:89-212)
  bool timing = false;
  bool no_fusion = false;  // force the per-routine kernels (tests compare both)
  bool no_tma = false;     // force the kernels without TMA staging (tests compare both)
  bool fct_fused = false;  // the three FCT stages as one kernel (with TMA)
  cudaEvent_t tev[6] = {};  // routine boundaries; [5]: the end of the fused path's iso-neutral fluxes
  double tms[4] = {0, 0, 0, 0};
  int tcalls = 0;
  // per-kernel timing (events after every launch while timing is on)
  KernelClock kc;
  LaunchShape shape;  // block heights chosen by nemo_gpu_autotune (0: the default)
  // host copies: uploads and downloads run on their own streams, each in call order
  // (one stream already saturates the host link each way), so the downloads of one
  // step overlap the uploads of the next; every field has the events of its last
  // upload and last download, so work waits only for the copies of the fields it
  // reads or writes
  static constexpr int NUP = 1, NDOWN = 1;
  cudaStream_t h2d[NUP] = {}, d2h[NDOWN] = {};
  cudaEvent_t ev_main = nullptr;            // the context stream's work so far
  cudaEvent_t ev_upf[NEMO_F_COUNT] = {};    // the last upload of each field
  cudaEvent_t ev_field[NEMO_F_COUNT] = {};  // the last download of each field
  bool upf_pending[NEMO_F_COUNT] = {};
  bool field_pending[NEMO_F_COUNT] = {};
  // the staging buffer of each uploaded field: an upload copies the host buffer into
  // it on the copy stream as soon as the buffer's previous contents have been copied
  // into the field, and the work that next reads the field (or a download of it)
  // makes that device copy on its own stream; so the next step's uploads do not wait
  // for this step's readers of the fields
  void* stage[NEMO_F_COUNT] = {};
  size_t stage_bytes[NEMO_F_COUNT] = {};
  cudaEvent_t ev_h2d[NEMO_F_COUNT] = {};  // the last host copy into the staging buffer
  bool stage_dirty[NEMO_F_COUNT] = {};    // staged data not yet copied into the field
  // the end of dyn_spg_ts in the last (staged) hot-path step: downloads of what
  // dyn_spg_ts writes wait only for it
  cudaEvent_t ev_spg_done = nullptr;
  bool spg_done_valid = false;
  // hot path: the iso-neutral fluxes run on a side stream beside dyn_spg_ts
  cudaStream_t side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  double kms[NEMO_K_COUNT] = {};
  int kcnt[NEMO_K_COUNT] = {};
};

namespace nemo {
thread_local KernelClock* t_kclock = nullptr;
thread_local const LaunchShape* t_shape = nullptr;
}

namespace {

int fail(nemo_ctx* c, int code, const char* fmt, ...) {
  if (c) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    c->err = buf;
  }
  return code;
}

int cuda_fail(nemo_ctx* c, cudaError_t e, const char* what) {
  return fail(c, NEMO_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define CK(expr, what)                                  \
  do {                                                  \
    cudaError_t e_ = (expr);                            \
    if (e_ != cudaSuccess) return cuda_fail(c, e_, what); \
  } while (0)

// The device copy of field id's staged upload into the field, on stream st: after
// the host copy into the staging buffer and the field's pending download (the copy
// overwrites the field); ev_upf marks its end.
int flush_stage(nemo_ctx* c, cudaStream_t st, int id) {
  if (!c->stage_dirty[id]) return NEMO_OK;
  CK(cudaStreamWaitEvent(st, c->ev_h2d[id], 0), "staged upload");
  if (c->field_pending[id]) CK(cudaStreamWaitEvent(st, c->ev_field[id], 0), "staged upload");
  CK(cudaMemcpyAsync(c->f[id], c->stage[id], c->stage_bytes[id], cudaMemcpyDeviceToDevice, st), "staged upload");
  CK(cudaEventRecord(c->ev_upf[id], st), "staged upload");
  c->stage_dirty[id] = false;
  c->upf_pending[id] = true;
  return NEMO_OK;
}

// Make stream st wait for the pending upload of field id (its device data) and, when
// `writes`, for its pending download (the work overwrites it).
int wait_field(nemo_ctx* c, cudaStream_t st, int id, bool writes) {
  if (flush_stage(c, st, id)) return NEMO_ERR_CUDA;
  if (c->upf_pending[id]) CK(cudaStreamWaitEvent(st, c->ev_upf[id], 0), "wait for an upload");
  if (writes && c->field_pending[id]) CK(cudaStreamWaitEvent(st, c->ev_field[id], 0), "wait for a download");
  return NEMO_OK;
}

// Before the context stream runs work: wait for every pending host copy (the work
// reads uploaded fields and may overwrite fields being downloaded).
int join_copies(nemo_ctx* c) {
  c->spg_done_valid = false;
  for (int id = 0; id < NEMO_F_COUNT; ++id) {
    if (wait_field(c, c->stream, id, true)) return NEMO_ERR_CUDA;
    c->upf_pending[id] = false;
    c->field_pending[id] = false;
  }
  return NEMO_OK;
}

bool copies_pending(const nemo_ctx* c) {
  for (int id = 0; id < NEMO_F_COUNT; ++id)
    if (c->upf_pending[id] || c->field_pending[id] || c->stage_dirty[id]) return true;
  return false;
}

// the fields dyn_spg_ts writes (the 3-D velocities and trends, the time-filter sums and
// restart fields)
bool spg_writes(int id) {
  switch (id) {
    case NEMO_F_UA: case NEMO_F_VA: case NEMO_F_UN: case NEMO_F_VN:
    case NEMO_F_SSHA: case NEMO_F_UA_B: case NEMO_F_VA_B: case NEMO_F_UN_ADV: case NEMO_F_VN_ADV:
    case NEMO_F_UB2_B: case NEMO_F_VB2_B: case NEMO_F_UN_BF: case NEMO_F_VN_BF:
      return true;
    default:
      return false;
  }
}
// the fields dyn_spg_ts reads besides those it writes: the before velocities, the
// scale factors at u- and v-points, every 2-D field (and e3f_n)
bool spg_reads(int id) {
  if (spg_writes(id) || id == NEMO_F_UB || id == NEMO_F_VB || id == NEMO_F_E3U_N || id == NEMO_F_E3V_N) return true;
  return id >= NEMO_F_SSHB && id < NEMO_F_FCT_TAPE;
}

inline size_t I2(const nemo_ctx* c, int i, int j) { return (size_t)(i - 1) + (size_t)c->jpi * (j - 1); }
inline size_t I3(const nemo_ctx* c, int i, int j, int k) { return I2(c, i, j) + (size_t)c->n2 * (k - 1); }

bool is_fp64_field(int id) {
  switch (id) {
    case NEMO_F_SSHA: case NEMO_F_UA_B: case NEMO_F_VA_B: case NEMO_F_UN_ADV: case NEMO_F_VN_ADV:
    case NEMO_F_UB2_B: case NEMO_F_VB2_B: case NEMO_F_UN_BF: case NEMO_F_VN_BF:
      return true;
    default:
      return false;
  }
}

size_t field_numel(const nemo_ctx* c, int id) {
  switch (id) {
    case NEMO_F_TSB: case NEMO_F_TSN: case NEMO_F_TSA: return 2 * (size_t)c->n3;
    case NEMO_F_GTSU: case NEMO_F_GTSV: case NEMO_F_GTUI: case NEMO_F_GTVI: return 2 * (size_t)c->n2;
    case NEMO_F_E3F_N: return (size_t)c->n3;
    case NEMO_F_FCT_TAPE: return 6 * (size_t)c->n3;  // 3 faces x 2 tracers
    case NEMO_F_GDEPT_N: case NEMO_F_GDEPW_N: return (size_t)c->n3;
    case NEMO_F_SBC_TSC: case NEMO_F_SBC_TSC_B: return 2 * (size_t)c->n2;
    case NEMO_F_QSR_HC: case NEMO_F_QSR_HC_B: return (size_t)c->n3;
    case NEMO_F_RHD: case NEMO_F_RHOP: case NEMO_F_RN2B: case NEMO_F_AHMT: case NEMO_F_AHMF: return (size_t)c->n3;
    case NEMO_F_AVM: case NEMO_F_AVM_K: case NEMO_F_AVT_K: case NEMO_F_EN: case NEMO_F_DISSL: case NEMO_F_RN2:
      return (size_t)c->n3;
    case NEMO_F_E3U_A: case NEMO_F_E3V_A: case NEMO_F_E3U_B: case NEMO_F_E3V_B: case NEMO_F_E3W_B:
    case NEMO_F_E3UW_N: case NEMO_F_E3VW_N: case NEMO_F_E3UW_B: case NEMO_F_E3VW_B:
    case NEMO_F_GDEPT_B: case NEMO_F_GDEPW_B: case NEMO_F_GDE3W_N: case NEMO_F_E3UW_0: case NEMO_F_E3VW_0:
    case NEMO_F_WSLP2:
      return (size_t)c->n3;
    case NEMO_F_TRIADI_G: case NEMO_F_TRIADJ_G: case NEMO_F_TRIADI: case NEMO_F_TRIADJ:
      return 4 * (size_t)c->n3;
    default: break;
  }
  if (id >= NEMO_F_SSHB) return (size_t)c->n2;
  return (size_t)c->n3;
}

// ts_wgt (dynspg_ts.F90:1313-1388)
void ts_wgt(nemo_ctx* c, int ll_av, int ll_fw, int* jpit) {
  const int nb = c->nn_baro, n3b = 3 * nb;
  c->wgt1.assign(n3b, 0.0);
  c->wgt2.assign(n3b, 0.0);
  int jic = ll_fw ? nb : 2 * nb;
  if (ll_av) {
    if (c->nam.nn_bt_flt == 0) {
      c->wgt1[jic - 1] = 1.0;
      *jpit = jic;
    } else {
      const double lim = c->nam.nn_bt_flt == 1 ? 0.5 : 1.0;
      for (int jn = 1; jn <= n3b; ++jn) {
        double za1 = std::fabs((double)(jn - jic)) / (double)nb;
        if (za1 < lim) { c->wgt1[jn - 1] = 1.0; *jpit = jn; }
      }
    }
  } else {
    c->wgt1[jic - 1] = 1.0;
    *jpit = jic;
  }
  for (int jn = 1; jn <= *jpit; ++jn)
    for (int ji = jn; ji <= *jpit; ++ji) c->wgt2[jn - 1] = c->wgt2[jn - 1] + c->wgt1[ji - 1];
  double s1 = 0, s2 = 0;
  for (int jn = 1; jn <= *jpit; ++jn) { s1 += c->wgt1[jn - 1]; s2 += c->wgt2[jn - 1]; }
  const double za1 = 1.0 / s1, za2 = 1.0 / s2;
  for (int jn = 1; jn <= *jpit; ++jn) {
    c->wgt1[jn - 1] = c->wgt1[jn - 1] * za1;
    c->wgt2[jn - 1] = c->wgt2[jn - 1] * za2;
  }
}

// Coriolis factors of dyn_spg_ts for a linear free surface (dynspg_ts.F90:241-342).
void coriolis_factors(nemo_ctx* c, const std::vector<double>& tmask, const std::vector<double>& umask) {
  const int jpi = c->jpi, jpj = c->jpj, jpk = c->jpk;
  const size_t n2 = c->n2;
  c->zwz.assign(n2, 0.0);
  c->ftne.assign(n2, 0.0); c->ftnw.assign(n2, 0.0); c->ftse.assign(n2, 0.0); c->ftsw.assign(n2, 0.0);
  const int sc = c->nam.nvor_scheme;
  const auto& ht = c->ht_0;
  const auto& ssm = c->ssmask;
  (void)tmask;
  if (sc == NEMO_VOR_EEN) {
    for (int jj = 1; jj <= jpj - 1; ++jj)
      for (int ji = 1; ji <= jpi - 1; ++ji) {
        double z;
        double s = ht[I2(c, ji, jj + 1)] + ht[I2(c, ji + 1, jj + 1)] + ht[I2(c, ji, jj)] + ht[I2(c, ji + 1, jj)];
        if (c->nam.nn_een_e3f == 0) z = s * 0.25;
        else {
          double m = ssm[I2(c, ji, jj + 1)] + ssm[I2(c, ji + 1, jj + 1)] + ssm[I2(c, ji, jj)] + ssm[I2(c, ji + 1, jj)];
          z = s / (m > 1.0 ? m : 1.0);
        }
        if (z != 0.0) z = c->ff_f[I2(c, ji, jj)] / z;
        c->zwz[I2(c, ji, jj)] = z;
      }
    for (int jj = 1; jj <= jpj; ++jj) c->zwz[I2(c, jpi, jj)] = 0.0;
    for (int ji = 1; ji <= jpi; ++ji) c->zwz[I2(c, ji, jpj)] = 0.0;
    const auto& w = c->zwz;
    for (int jj = 2; jj <= jpj; ++jj)
      for (int ji = 2; ji <= jpi; ++ji) {
        c->ftne[I2(c, ji, jj)] = w[I2(c, ji - 1, jj)] + w[I2(c, ji, jj)] + w[I2(c, ji, jj - 1)];
        c->ftnw[I2(c, ji, jj)] = w[I2(c, ji - 1, jj - 1)] + w[I2(c, ji - 1, jj)] + w[I2(c, ji, jj)];
        c->ftse[I2(c, ji, jj)] = w[I2(c, ji, jj)] + w[I2(c, ji, jj - 1)] + w[I2(c, ji - 1, jj - 1)];
        c->ftsw[I2(c, ji, jj)] = w[I2(c, ji, jj - 1)] + w[I2(c, ji - 1, jj - 1)] + w[I2(c, ji - 1, jj)];
      }
  } else if (sc == NEMO_VOR_EET) {
    const auto& ff = c->ff_f;
    for (int jj = 2; jj <= jpj; ++jj)
      for (int ji = 2; ji <= jpi; ++ji) {
        double z1_ht = ssm[I2(c, ji, jj)] / (ht[I2(c, ji, jj)] + 1.0 - ssm[I2(c, ji, jj)]);
        c->ftne[I2(c, ji, jj)] = (ff[I2(c, ji - 1, jj)] + ff[I2(c, ji, jj)] + ff[I2(c, ji, jj - 1)]) * z1_ht;
        c->ftnw[I2(c, ji, jj)] = (ff[I2(c, ji - 1, jj - 1)] + ff[I2(c, ji - 1, jj)] + ff[I2(c, ji, jj)]) * z1_ht;
        c->ftse[I2(c, ji, jj)] = (ff[I2(c, ji, jj)] + ff[I2(c, ji, jj - 1)] + ff[I2(c, ji - 1, jj - 1)]) * z1_ht;
        c->ftsw[I2(c, ji, jj)] = (ff[I2(c, ji, jj - 1)] + ff[I2(c, ji - 1, jj - 1)] + ff[I2(c, ji - 1, jj)]) * z1_ht;
      }
  } else if (sc == NEMO_VOR_ENE || sc == NEMO_VOR_ENS || sc == NEMO_VOR_MIX) {
    std::vector<double> zhf(n2, 0.0);
    if (c->nam.ln_sco)
      for (int jj = 1; jj <= jpj - 1; ++jj)
        for (int ji = 1; ji <= jpi - 1; ++ji) {
          double m = ssm[I2(c, ji, jj)] + ssm[I2(c, ji + 1, jj)] + ssm[I2(c, ji, jj + 1)] + ssm[I2(c, ji + 1, jj + 1)];
          zhf[I2(c, ji, jj)] = (ht[I2(c, ji, jj)] + ht[I2(c, ji + 1, jj)] + ht[I2(c, ji, jj + 1)] + ht[I2(c, ji + 1, jj + 1)]) /
                               (m > 1.0 ? m : 1.0);
        }
    for (int jj = 1; jj <= jpj - 1; ++jj)
      for (int ji = 1; ji <= jpi; ++ji)
        zhf[I2(c, ji, jj)] = zhf[I2(c, ji, jj)] * (1.0 - umask[I3(c, ji, jj, 1)] * umask[I3(c, ji, jj + 1, 1)]);
    for (int jk = 1; jk <= jpk - 1; ++jk)
      for (int jj = 1; jj <= jpj - 1; ++jj)
        for (int ji = 1; ji <= jpi; ++ji)
          zhf[I2(c, ji, jj)] =
              zhf[I2(c, ji, jj)] + c->e3_0[4][I3(c, ji, jj, jk)] * umask[I3(c, ji, jj, jk)] * umask[I3(c, ji, jj + 1, jk)];
    for (int jj = 1; jj <= jpj; ++jj) zhf[I2(c, jpi, jj)] = 0.0;
    for (int ji = 1; ji <= jpi; ++ji) zhf[I2(c, ji, jpj)] = 0.0;
    for (size_t p = 0; p < n2; ++p)
      if (zhf[p] != 0.0) c->zwz[p] = 1.0 / zhf[p];
    for (size_t p = 0; p < n2; ++p) c->zwz[p] = c->ff_f[p] * c->zwz[p];
  }
}

template <class T>
int upload(nemo_ctx* c, DomStore<T>& st, const std::vector<double>& src, RO<T>* dst) {
  std::vector<T> h(src.size());
  for (size_t i = 0; i < src.size(); ++i) h[i] = (T)src[i];
  void* p = nullptr;
  CK(cudaMalloc(&p, h.size() * sizeof(T) + 16), "cudaMalloc(domain)");
  st.owned.push_back(p);
  CK(cudaMemcpy(p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice), "upload(domain)");
  *dst = (const T*)p;
  return NEMO_OK;
}

// e3 field: a 1-D profile when horizontally uniform, else the full 3-D array.
template <class T>
int upload_e3(nemo_ctx* c, DomStore<T>& st, int which, E3<T>* e) {
  const auto& a = c->e3_0[which];
  if (c->e3_uniform[which]) {
    std::vector<double> prof(c->jpk);
    for (int k = 0; k < c->jpk; ++k) prof[k] = a[(size_t)k * c->n2];
    RO<T> p;
    int st_ = upload(c, st, prof, &p);
    if (st_) return st_;
    *e = E3<T>{p, 1, 0, 0};
  } else {
    RO<T> p;
    int st_ = upload(c, st, a, &p);
    if (st_) return st_;
    *e = E3<T>{p, c->n2, 0, 1};
  }
  return NEMO_OK;
}

template <class T>
int build_dom(nemo_ctx* c, DomStore<T>& st) {
  Dom<T>& d = st.d;
  d.jpi = c->jpi; d.jpj = c->jpj; d.jpk = c->jpk; d.nmem = c->nmem; d.n2 = c->n2; d.n3 = c->n3;
  int s = 0;
#define UP(name) if ((s = upload(c, st, c->name, &d.name))) return s
  UP(e1t); UP(e2t); UP(e1u); UP(e2u); UP(e1v); UP(e2v);
  UP(r1_e1u); UP(r1_e2u); UP(r1_e1v); UP(r1_e2v);
  UP(e1e2t); UP(r1_e1e2t); UP(e2_e1u); UP(e1_e2v); UP(r1_e1e2u); UP(r1_e1e2v); UP(r1_e1e2f); UP(e1e2u); UP(e1e2v);
  UP(ht_0); UP(hu_0); UP(hv_0); UP(r1_hu_0); UP(r1_hv_0);
  UP(ssmask); UP(ssumask); UP(ssvmask);
  UP(ff_t); UP(ff_f); UP(zwz); UP(ftne); UP(ftnw); UP(ftse); UP(ftsw);
#undef UP
  {
    void* p = nullptr;
    CK(cudaMalloc(&p, c->n2 * sizeof(double)), "cudaMalloc(tmask_i)");
    st.owned.push_back(p);
    CK(cudaMemcpy(p, c->tmask_i.data(), c->n2 * sizeof(double), cudaMemcpyHostToDevice), "upload(tmask_i)");
    d.tmask_i = (const double*)p;
    CK(cudaMalloc(&p, c->n2 * sizeof(ColInfo)), "cudaMalloc(colinfo)");
    st.owned.push_back(p);
    CK(cudaMemcpy(p, c->ci.data(), c->n2 * sizeof(ColInfo), cudaMemcpyHostToDevice), "upload(colinfo)");
    d.ci = (const ColInfo*)p;
    CK(cudaMalloc(&p, c->n2), "cudaMalloc(mbkt)");
    st.owned.push_back(p);
    CK(cudaMemcpy(p, c->mbkt.data(), c->n2, cudaMemcpyHostToDevice), "upload(mbkt)");
    d.mbkt = (const uint8_t*)p;
  }
  if ((s = upload_e3(c, st, 0, &d.e3t_n))) return s;
  d.e3t_b = d.e3t_n; d.e3t_a = d.e3t_n;
  if ((s = upload_e3(c, st, 1, &d.e3u_n))) return s;
  if ((s = upload_e3(c, st, 2, &d.e3v_n))) return s;
  if ((s = upload_e3(c, st, 3, &d.e3w_n))) return s;
  if ((s = upload_e3(c, st, 4, &d.e3f_n))) return s;
  for (int w : {0, 3}) {  // reciprocal profiles of e3t_0 and e3w_0
    if (!c->e3_uniform[w]) continue;
    std::vector<double> r(c->jpk);
    for (int k = 0; k < c->jpk; ++k) r[k] = 1.0 / c->e3_0[w][(size_t)k * c->n2];
    if ((s = upload(c, st, r, w == 0 ? &d.r1_e3t : &d.r1_e3w))) return s;
  }
  return NEMO_OK;
}

template <class T>
void free_dom(DomStore<T>& st) {
  for (void* p : st.owned) cudaFree(p);
  st.owned.clear();
}

// The sub-step weights as the mixed form's sub-step kernel uses them: wgt1 = hi + lo
// (two floats, for the compensated sums) and wgt2 rounded to float, in three blocks
// of wgt1.size() entries.
void float_weights(nemo_ctx* c) {
  const size_t n = c->wgt1.size();
  c->wgtf.assign(3 * n, 0.0f);
  for (size_t i = 0; i < n; ++i) {
    const float h = (float)c->wgt1[i];
    c->wgtf[i] = h;
    c->wgtf[n + i] = (float)(c->wgt1[i] - (double)h);
    c->wgtf[2 * n + i] = (float)c->wgt2[i];
  }
}

// trc_oce_ext_lev (trc_oce.F90:215-256): the last T-level reached by a fraction
// pqsr_frc of the light of longest extinction depth prldex, or the sea bed; the
// rest-state W-depths are the sums of e3t_0 of e3_to_depth (DOM/depth_e3.F90).
int ext_lev(const nemo_ctx* c, double prldex, double pqsr_frc) {
  const int jpk = c->jpk;
  const size_t n2 = c->n2;
  const double zhext = prldex * (std::log(10.0) * 15.0 + std::log(pqsr_frc));
  std::vector<double> gdepw((size_t)jpk * n2, 0.0);
  for (int jk = 2; jk <= jpk; ++jk)
    for (size_t p = 0; p < n2; ++p)
      gdepw[p + n2 * (jk - 1)] = gdepw[p + n2 * (jk - 2)] + c->e3_0[0][p + n2 * (jk - 2)];
  int pjl = jpk - 1;
  for (int jk = jpk - 1; jk >= 1; --jk) {
    bool wet = false;
    double zem = -1e300;
    for (size_t p = 0; p < n2; ++p) {
      const double tm = (jk >= c->ci[p].tlo && jk <= c->ci[p].thi) ? 1.0 : 0.0;
      wet = wet || tm > 0;
      zem = std::max(zem, gdepw[p + n2 * jk] * tm);
    }
    if (!wet || zem >= zhext) pjl = jk;
  }
  return pjl;
}

// nlb10 (domzgr.F90:144-146): the shallowest W-level deeper than 10 m less a tenth
// of the thinnest W-layer, on the 1-D reference profile (the rest-state column with
// the most wet levels; gdepw_1d from its e3t_0 as e3_to_depth sums them).
int nlb10_of(const nemo_ctx* c) {
  const size_t n2 = c->n2;
  size_t best = 0;
  for (size_t p = 0; p < n2; ++p)
    if (c->mbkt[p] > c->mbkt[best]) best = p;
  double e3wmin = 1e300, gdepw = 0.0;
  for (int jk = 1; jk <= c->jpk; ++jk) e3wmin = std::min(e3wmin, c->e3_0[3][best + n2 * (jk - 1)]);
  const double zrefdep = 10.0 - 0.1 * e3wmin;
  for (int jk = 1; jk <= c->jpk; ++jk) {
    if (gdepw > zrefdep) return jk;
    gdepw = gdepw + c->e3_0[0][best + n2 * (jk - 1)];
  }
  return c->jpk;
}

// Domain derivation (dommsk.F90:133-238, domzgr.F90:292-314, domhgr.F90:133-151,
// domain.F90:149-183) and spg set-up (dynspg_ts.F90:1479-1493).
int derive_domain(nemo_ctx* c, const nemo_dom_desc* dm) {
  const int jpi = c->jpi, jpj = c->jpj, jpk = c->jpk;
  const size_t n2 = c->n2, n3 = c->n3;
  auto cp2 = [&](std::vector<double>& v, const double* s) { v.assign(s, s + n2); };
  cp2(c->e1t, dm->e1t); cp2(c->e2t, dm->e2t); cp2(c->e1u, dm->e1u); cp2(c->e2u, dm->e2u);
  cp2(c->e1v, dm->e1v); cp2(c->e2v, dm->e2v); cp2(c->e1f, dm->e1f); cp2(c->e2f, dm->e2f);
  cp2(c->ff_f, dm->ff_f); cp2(c->ff_t, dm->ff_t);
  const double* e3s[5] = {dm->e3t_0, dm->e3u_0, dm->e3v_0, dm->e3w_0, dm->e3f_0};
  for (int w = 0; w < 5; ++w) {
    c->e3_0[w].assign(e3s[w], e3s[w] + n3);
    bool uni = true;
    for (int k = 0; k < jpk && uni; ++k) {
      const double v0 = c->e3_0[w][(size_t)k * n2];
      for (size_t p = 0; p < n2; ++p)
        if (c->e3_0[w][(size_t)k * n2 + p] != v0) { uni = false; break; }
    }
    c->e3_uniform[w] = uni;
  }
  auto mk = [&](std::vector<double>& v) { v.assign(n2, 0.0); };
  mk(c->r1_e1t); mk(c->r1_e2t); mk(c->r1_e1u); mk(c->r1_e2u); mk(c->r1_e1v); mk(c->r1_e2v); mk(c->e1e2t);
  mk(c->r1_e1e2t); mk(c->e1e2u); mk(c->e1e2v); mk(c->r1_e1e2u); mk(c->r1_e1e2v); mk(c->e2_e1u); mk(c->e1_e2v); mk(c->r1_e1e2f);
  for (size_t p = 0; p < n2; ++p) {
    c->r1_e1t[p] = 1.0 / c->e1t[p]; c->r1_e2t[p] = 1.0 / c->e2t[p];
    c->r1_e1u[p] = 1.0 / c->e1u[p]; c->r1_e2u[p] = 1.0 / c->e2u[p];
    c->r1_e1v[p] = 1.0 / c->e1v[p]; c->r1_e2v[p] = 1.0 / c->e2v[p];
    c->e1e2t[p] = c->e1t[p] * c->e2t[p]; c->r1_e1e2t[p] = 1.0 / c->e1e2t[p];
    c->e1e2u[p] = c->e1u[p] * c->e2u[p]; c->e1e2v[p] = c->e1v[p] * c->e2v[p];
    c->r1_e1e2u[p] = 1.0 / c->e1e2u[p]; c->r1_e1e2v[p] = 1.0 / c->e1e2v[p];
    c->r1_e1e2f[p] = 1.0 / (c->e1f[p] * c->e2f[p]);
    c->e2_e1u[p] = c->e2u[p] / c->e1u[p]; c->e1_e2v[p] = c->e1v[p] / c->e2v[p];
  }
  // masks
  std::vector<double> tmask(n3, 0.0), umask(n3, 0.0), vmask(n3, 0.0);
  for (int jj = 1; jj <= jpj; ++jj)
    for (int ji = 1; ji <= jpi; ++ji) {
      int kt = dm->k_top[I2(c, ji, jj)], kb = dm->k_bot[I2(c, ji, jj)];
      if (kt < 0 || kt > 1) return fail(c, NEMO_ERR_UNSUPPORTED, "k_top(%d,%d)=%d: ice-shelf cavities are not supported", ji, jj, kt);
      if (kb < 0 || kb > jpk) return fail(c, NEMO_ERR_ARG, "k_bot(%d,%d)=%d out of range", ji, jj, kb);
      bool edge = ji == 1 || ji == jpi || jj == 1 || jj == jpj;
      if (kt != 0 && !edge)
        for (int jk = kt; jk <= kb; ++jk) tmask[I3(c, ji, jj, jk)] = 1.0;
    }
  for (int jk = 1; jk <= jpk; ++jk)
    for (int jj = 1; jj <= jpj - 1; ++jj)
      for (int ji = 1; ji <= jpi - 1; ++ji) {
        umask[I3(c, ji, jj, jk)] = tmask[I3(c, ji, jj, jk)] * tmask[I3(c, ji + 1, jj, jk)];
        vmask[I3(c, ji, jj, jk)] = tmask[I3(c, ji, jj, jk)] * tmask[I3(c, ji, jj + 1, jk)];
      }
  for (int jk = 1; jk <= jpk; ++jk) {
    for (int jj = 1; jj <= jpj; ++jj) {
      umask[I3(c, 1, jj, jk)] = 0; umask[I3(c, jpi, jj, jk)] = 0;
      vmask[I3(c, 1, jj, jk)] = 0; vmask[I3(c, jpi, jj, jk)] = 0;
    }
    for (int ji = 1; ji <= jpi; ++ji) {
      umask[I3(c, ji, 1, jk)] = 0; umask[I3(c, ji, jpj, jk)] = 0;
      vmask[I3(c, ji, 1, jk)] = 0; vmask[I3(c, ji, jpj, jk)] = 0;
    }
  }
  // column ranges; verify that each mask is one contiguous level range
  c->ci.assign(n2, ColInfo{});
  c->mbkt.assign(n2, 1);
  auto range = [&](const std::vector<double>& m, size_t p, uint8_t& lo, uint8_t& hi) -> bool {
    int l = 0, h = -1;
    for (int k = 1; k <= jpk; ++k)
      if (m[p + n2 * (k - 1)] != 0.0) { if (l == 0) l = k; h = k; }
    if (l == 0) { lo = 1; hi = 0; return true; }
    for (int k = l; k <= h; ++k)
      if (m[p + n2 * (k - 1)] == 0.0) return false;
    lo = (uint8_t)l; hi = (uint8_t)h;
    return true;
  };
  for (size_t p = 0; p < n2; ++p) {
    ColInfo& q = c->ci[p];
    if (!range(tmask, p, q.tlo, q.thi) || !range(umask, p, q.ulo, q.uhi) || !range(vmask, p, q.vlo, q.vhi))
      return fail(c, NEMO_ERR_UNSUPPORTED, "column %zu: wet levels are not contiguous", p);
    int kb = dm->k_bot[p];
    c->mbkt[p] = (uint8_t)(kb > 1 ? kb : 1);
  }
  for (int jj = 1; jj <= jpj; ++jj)
    for (int ji = 1; ji <= jpi; ++ji) {
      ColInfo& q = c->ci[I2(c, ji, jj)];
      if (ji == jpi || jj == jpj || ji == 1 || jj == 1) { q.mbku = 1; q.mbkv = 1; continue; }
      int a = c->mbkt[I2(c, ji + 1, jj)], b = c->mbkt[I2(c, ji, jj)], e = c->mbkt[I2(c, ji, jj + 1)];
      q.mbku = (uint8_t)((a < b ? a : b) > 1 ? (a < b ? a : b) : 1);
      q.mbkv = (uint8_t)((e < b ? e : b) > 1 ? (e < b ? e : b) : 1);
    }
  c->ssmask.assign(n2, 0.0); c->ssumask.assign(n2, 0.0); c->ssvmask.assign(n2, 0.0); c->tmask_i.assign(n2, 0.0);
  for (size_t p = 0; p < n2; ++p) {
    const ColInfo& q = c->ci[p];
    c->ssmask[p] = q.tlo <= q.thi ? 1.0 : 0.0;
    c->ssumask[p] = q.ulo <= q.uhi ? 1.0 : 0.0;
    c->ssvmask[p] = q.vlo <= q.vhi ? 1.0 : 0.0;
  }
  for (int jj = 1; jj <= jpj; ++jj)
    for (int ji = 1; ji <= jpi; ++ji) {
      bool edge = ji == 1 || ji == jpi || jj == 1 || jj == jpj;
      c->tmask_i[I2(c, ji, jj)] = c->ssmask[I2(c, ji, jj)] * (edge ? 0.0 : 1.0);
    }
  c->ht_0.assign(n2, 0.0); c->hu_0.assign(n2, 0.0); c->hv_0.assign(n2, 0.0);
  c->r1_hu_0.assign(n2, 0.0); c->r1_hv_0.assign(n2, 0.0);
  for (int jk = 0; jk < jpk; ++jk)
    for (size_t p = 0; p < n2; ++p) {
      c->ht_0[p] = c->ht_0[p] + c->e3_0[0][p + n2 * jk] * tmask[p + n2 * jk];
      c->hu_0[p] = c->hu_0[p] + c->e3_0[1][p + n2 * jk] * umask[p + n2 * jk];
      c->hv_0[p] = c->hv_0[p] + c->e3_0[2][p + n2 * jk] * vmask[p + n2 * jk];
    }
  for (size_t p = 0; p < n2; ++p) {
    c->r1_hu_0[p] = c->ssumask[p] / (c->hu_0[p] + 1.0 - c->ssumask[p]);
    c->r1_hv_0[p] = c->ssvmask[p] / (c->hv_0[p] + 1.0 - c->ssvmask[p]);
  }
  // dyn_spg_ts_init
  double zcmax = -1e300;
  for (size_t p = 0; p < n2; ++p) {
    double zxr2 = c->r1_e1t[p] * c->r1_e1t[p], zyr2 = c->r1_e2t[p] * c->r1_e2t[p];
    double h = c->ht_0[p] > 0.0 ? c->ht_0[p] : 0.0;
    double zcu = std::sqrt(c->nam.grav * h * (zxr2 + zyr2));
    if (zcu > zcmax) zcmax = zcu;
  }
  c->nn_baro = c->nam.ln_bt_auto ? (int)std::ceil(c->nam.rn_rdt / c->nam.rn_bt_cmax * zcmax) : c->nam.nn_baro;
  if (c->nn_baro < 1) c->nn_baro = 1;
  c->rdtbt = c->nam.rn_rdt / (double)c->nn_baro;
  int jpit = 0;
  ts_wgt(c, c->nam.ln_bt_av, c->nam.ln_bt_fw, &jpit);
  c->icycle = jpit;
  c->nksr = ext_lev(c, c->nam.rn_si1 > 0 ? c->nam.rn_si1 : 23.0, 100.0);
  c->nlb10 = nlb10_of(c);
  coriolis_factors(c, tmask, umask);
  return NEMO_OK;
}

template <class T>
const Dom<T>& dom(nemo_ctx* c);
template <>
const Dom<double>& dom<double>(nemo_ctx* c) { return c->dd.d; }
template <>
const Dom<float>& dom<float>(nemo_ctx* c) { return c->df.d; }

// Dom with the bound time-varying e3 fields substituted for the rest state.
template <class T>
Dom<T> dom_now(nemo_ctx* c) {
  Dom<T> d = dom<T>(c);
  auto sub = [&](int id, E3<T>& e) {
    if (c->f[id]) e = E3<T>{(const T*)c->f[id], c->n2, c->n3, 1};
  };
  sub(NEMO_F_E3T_B, d.e3t_b); sub(NEMO_F_E3T_N, d.e3t_n); sub(NEMO_F_E3T_A, d.e3t_a);
  sub(NEMO_F_E3U_N, d.e3u_n); sub(NEMO_F_E3V_N, d.e3v_n); sub(NEMO_F_E3W_N, d.e3w_n);
  sub(NEMO_F_E3F_N, d.e3f_n);
  return d;
}

int ensure_fct_work(nemo_ctx* c, int kjpt, int need_ztw) {
  const size_t es = c->prec == NEMO_PREC_FP64 ? 8 : 4;
  const size_t bytes = (size_t)kjpt * c->n3 * c->nmem * es;
  if (kjpt > c->fct_kjpt) {
    for (auto& p : c->fct_w) { cudaFree(p); p = nullptr; }
    cudaFree(c->fct_ztw); c->fct_ztw = nullptr;
    for (auto& p : c->fct_w) {
      if (cudaMalloc(&p, bytes) != cudaSuccess) return fail(c, NEMO_ERR_NOMEM, "FCT work arrays (%zu bytes)", bytes);
      cudaMemset(p, 0, bytes);
    }
    c->fct_kjpt = kjpt;
  }
  if (need_ztw && !c->fct_ztw) {
    if (cudaMalloc(&c->fct_ztw, (size_t)c->fct_kjpt * c->n3 * c->nmem * es) != cudaSuccess)
      return fail(c, NEMO_ERR_NOMEM, "FCT compact-interpolation array");
    cudaMemset(c->fct_ztw, 0, (size_t)c->fct_kjpt * c->n3 * c->nmem * es);
  }
  return NEMO_OK;
}

int ensure_iso_work(nemo_ctx* c, int kjpt) {
  if (kjpt <= c->iso_kjpt) return NEMO_OK;
  const size_t bytes = (size_t)kjpt * c->n3 * c->nmem * (c->prec == NEMO_PREC_FP64 ? 8 : 4);
  for (auto& p : c->iso_w) {
    cudaFree(p);
    p = nullptr;
  }
  for (auto& p : c->iso_w)
    if (cudaMalloc(&p, bytes) != cudaSuccess) return fail(c, NEMO_ERR_NOMEM, "iso-neutral flux arrays (%zu bytes)", bytes);
  c->iso_kjpt = kjpt;
  return NEMO_OK;
}

int check_cdtype(nemo_ctx* c, const char* cdtype, int* is_trc) {
  if (!cdtype) return fail(c, NEMO_ERR_ARG, "cdtype is NULL");
  if (!strncmp(cdtype, "TRA", 3)) *is_trc = 0;
  else if (!strncmp(cdtype, "TRC", 3)) *is_trc = 1;
  else return fail(c, NEMO_ERR_ARG, "cdtype must be TRA or TRC");
  return NEMO_OK;
}

template <class T>
int run_fct(nemo_ctx* c, double p2dt, const void* pun, const void* pvn, const void* pwn, int trp, const void* ptb,
            const void* ptn, const void* pta_in, void* pta, int kjpt, int kh, int kv,
            const LdfArgs<T>* iso = nullptr, void* lim = nullptr) {
  int s = ensure_fct_work(c, kjpt, kv == 4);
  if (s) return s;
  FctArgs<T> a{};
  if (lim) {  // record the limiter multipliers (0 on the faces the forward zeroes)
    a.lim = (T*)lim;
    CK(cudaMemsetAsync(lim, 0, 3 * (size_t)kjpt * c->n3 * c->nmem * sizeof(T), c->stream), "FCT tape = 0");
  }
  a.p2dt = (T)p2dt;
  a.r1_p2dt = (T)(1.0 / p2dt);
  a.pun = (const T*)pun; a.pvn = (const T*)pvn; a.pwn = (const T*)pwn; a.trp = trp;
  a.ptb = (const T*)ptb; a.ptn = (const T*)ptn; a.pta_in = (const T*)pta_in; a.pta = (T*)pta;
  a.zwi = (T*)c->fct_w[0]; a.ax = (T*)c->fct_w[1]; a.ay = (T*)c->fct_w[2]; a.az = (T*)c->fct_w[3];
  a.betup = (T*)c->fct_w[4]; a.betdo = (T*)c->fct_w[5];
  a.ztw = (const T*)c->fct_ztw;
  a.kjpt = kjpt; a.kn_fct_h = kh; a.kn_fct_v = kv; a.linssh = c->nam.ln_linssh;
  a.tma = !c->no_tma; a.fused = c->fct_fused; a.err = c->err_flag; a.polls = c->tma_polls;
  if (iso) {
    a.with_iso = 1;
    a.iso = *iso;
  }
  cudaError_t e = launch_fct<T>(dom_now<T>(c), a, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "tra_adv_fct launch");
  return NEMO_OK;
}

template <class T>
LdfArgs<T> ldf_args(nemo_ctx* c, const void* pahu, const void* pahv, const void* pgu, const void* pgv, const void* ptb,
                    const void* ptbb, void* pta, int kjpt, int kpass) {
  LdfArgs<T> a{};
  a.pahu = (const T*)pahu; a.pahv = (const T*)pahv;
  a.aht_c = (T)(c->nam.ln_traldf_blp ? std::sqrt(c->nam.rn_aht_0) : c->nam.rn_aht_0);
  a.pgu = (const T*)pgu; a.pgv = (const T*)pgv; a.zps = c->nam.ln_zps;
  a.ptb = (const T*)ptb; a.ptbb = (const T*)ptbb; a.pta = (T*)pta;
  a.kjpt = kjpt; a.kpass = kpass; a.zsign = kpass == 1 ? T(1) : T(-1);
  return a;
}

template <class T>
int run_ldf_lap(nemo_ctx* c, const void* pahu, const void* pahv, const void* pgu, const void* pgv, const void* ptb,
                void* pta, int kjpt, int kpass) {
  LdfArgs<T> a = ldf_args<T>(c, pahu, pahv, pgu, pgv, ptb, ptb, pta, kjpt, kpass);
  cudaError_t e = launch_ldf_lap<T>(dom_now<T>(c), a, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "tra_ldf_lap launch");
  return NEMO_OK;
}

// Iso-neutral arguments for one call (traldf_iso.F90:130-203): bound slopes and
// coefficient arrays, time step, and on the first pass of kit000 the zeroing of
// ah_wslp2 / akz.
template <class T>
int iso_args(nemo_ctx* c, int kt, int kit000, const void* pahu, const void* pahv, const void* pgu, const void* pgv,
             const void* ptb, const void* ptbb, void* pta, int kjpt, int kpass, LdfArgs<T>* out) {
  const nemo_namelist& nm = c->nam;
  if (!c->f[NEMO_F_USLP] || !c->f[NEMO_F_VSLP] || !c->f[NEMO_F_WSLPI] || !c->f[NEMO_F_WSLPJ] ||
      !c->f[NEMO_F_AH_WSLP2] || !c->f[NEMO_F_AKZ])
    return fail(c, NEMO_ERR_UNBOUND, "tra_ldf_iso: slopes, ah_wslp2 and akz must be bound");
  int s = ensure_iso_work(c, kjpt);
  if (s) return s;
  LdfArgs<T> a = ldf_args<T>(c, pahu, pahv, pgu, pgv, ptb, ptbb, pta, kjpt, kpass);
  a.uslp = (const T*)c->f[NEMO_F_USLP]; a.vslp = (const T*)c->f[NEMO_F_VSLP];
  a.wslpi = (const T*)c->f[NEMO_F_WSLPI]; a.wslpj = (const T*)c->f[NEMO_F_WSLPJ];
  a.ah_wslp2 = (T*)c->f[NEMO_F_AH_WSLP2]; a.akz = (T*)c->f[NEMO_F_AKZ];
  a.lap = nm.ln_traldf_lap; a.blp = nm.ln_traldf_blp; a.msc = nm.ln_traldf_msc;
  a.zftu = (T*)c->iso_w[0]; a.zftv = (T*)c->iso_w[1]; a.ztfw = (T*)c->iso_w[2];
  a.tma = !c->no_tma; a.err = c->err_flag; a.polls = c->tma_polls;
  const double z2dt = (nm.neuler == 0 && kt == nm.nit000) ? nm.rn_rdt : 2.0 * nm.rn_rdt;
  a.z2dt = (T)z2dt; a.z1_2dt = (T)(1.0 / z2dt);
  if (kpass == 1 && kt == kit000) {
    const size_t bytes = c->n3 * c->nmem * sizeof(T);
    CK(cudaMemsetAsync(a.akz, 0, bytes, c->stream), "akz = 0");
    CK(cudaMemsetAsync(a.ah_wslp2, 0, bytes, c->stream), "ah_wslp2 = 0");
  }
  *out = a;
  return NEMO_OK;
}

template <class T>
int run_ldf_iso(nemo_ctx* c, int kt, int kit000, const void* pahu, const void* pahv, const void* pgu, const void* pgv,
                const void* ptb, const void* ptbb, void* pta, int kjpt, int kpass) {
  LdfArgs<T> a{};
  int s = iso_args<T>(c, kt, kit000, pahu, pahv, pgu, pgv, ptb, ptbb, pta, kjpt, kpass, &a);
  if (s) return s;
  const nemo_namelist& nm = c->nam;
  cudaError_t e = launch_ldf_iso<T>(dom_now<T>(c), a, kpass == 1 && !nm.ln_traldf_msc,
                                    kpass == 1 && nm.ln_traldf_msc, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "tra_ldf_iso launch");
  return NEMO_OK;
}

// tra_ldf_blp (traldf_lap_blp.F90:161-231) without partial steps: the first
// laplacian (kldf 20 iso-level, 21 rotated) of ptb into zlap, lbc_lnk, the second of
// zlap into pta
// ---------------------------------------------------------------- the triad operator
template <class T>
TriadArgs<T> triad_args(nemo_ctx* c) {
  const nemo_namelist& nm = c->nam;
  void* const* F = c->f;
  TriadArgs<T> a{};
  a.tsb = (const T*)F[NEMO_F_TSB];
  a.gdept = (const T*)F[NEMO_F_GDEPT_N]; a.gdepw = (const T*)F[NEMO_F_GDEPW_N];
  a.nmln = (const int*)F[NEMO_F_NMLN];
  a.tig = (T*)F[NEMO_F_TRIADI_G]; a.tjg = (T*)F[NEMO_F_TRIADJ_G]; a.ti = (T*)F[NEMO_F_TRIADI]; a.tj = (T*)F[NEMO_F_TRIADJ];
  a.wslp2 = (T*)F[NEMO_F_WSLP2];
  a.slpmax = (T)(nm.rn_slpmax > 0 ? nm.rn_slpmax : 0.01);
  a.sw = (T)nm.rn_sw_triad;
  a.repsln = (T)1.e-25;   // ldfslp.F90:72
  a.triad_iso = nm.ln_triad_iso;
  a.botmix = nm.ln_botmix_triad;
  return a;
}

template <class T>
int run_ldf_triad(nemo_ctx* c, int kt, int kit000, const void* pahu, const void* pahv, const void* ptb,
                  const void* ptbb, void* pta, int kjpt, int kpass) {
  const nemo_namelist& nm = c->nam;
  if (int s = ensure_iso_work(c, kjpt)) return s;
  TriadArgs<T> a = triad_args<T>(c);
  a.l = ldf_args<T>(c, pahu, pahv, nullptr, nullptr, ptb, ptbb, pta, kjpt, kpass);
  a.l.ah_wslp2 = (T*)c->f[NEMO_F_AH_WSLP2]; a.l.akz = (T*)c->f[NEMO_F_AKZ];
  a.l.lap = nm.ln_traldf_lap; a.l.blp = nm.ln_traldf_blp; a.l.msc = nm.ln_traldf_msc;
  const double z2dt = (nm.neuler == 0 && kt == kit000) ? nm.rn_rdt : 2.0 * nm.rn_rdt;  // traldf_triad.F90:117-120
  a.l.z2dt = (T)z2dt; a.l.z1_2dt = (T)(1.0 / z2dt);
  a.l.zftu = (T*)c->iso_w[0]; a.l.zftv = (T*)c->iso_w[1]; a.l.ztfw = (T*)c->iso_w[2];
  cudaError_t e = launch_tra_ldf_triad<T>(dom_now<T>(c), a, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "tra_ldf_triad launch");
  return NEMO_OK;
}

template <class T>
int run_ldf_blp(nemo_ctx* c, int kt, int kit000, const void* pahu, const void* pahv, const void* pgu,
                const void* pgv, const void* ptb, void* pta, int kjpt, int kldf) {
  const size_t n3b = (size_t)kjpt * c->n3 * c->nmem * sizeof(T), n2b = (size_t)kjpt * c->n2 * c->nmem * sizeof(T);
  if (kjpt > c->blp_kjpt) {
    cudaFree(c->blp_w);
    c->blp_w = nullptr;
    if (cudaMalloc(&c->blp_w, n3b + 2 * n2b) != cudaSuccess) return fail(c, NEMO_ERR_NOMEM, "tra_ldf_blp work array");
    c->blp_kjpt = kjpt;
  }
  T* zlap = (T*)c->blp_w;
  T* zglu = (T*)((char*)c->blp_w + n3b);
  T* zglv = (T*)((char*)c->blp_w + n3b + n2b);
  CK(cudaMemsetAsync(zlap, 0, n3b, c->stream), "zlap = 0");
  int s = kldf == 20 ? run_ldf_lap<T>(c, pahu, pahv, pgu, pgv, ptb, zlap, kjpt, 1)
          : kldf == 21 ? run_ldf_iso<T>(c, kt, kit000, pahu, pahv, pgu, pgv, ptb, ptb, zlap, kjpt, 1)
                       : run_ldf_triad<T>(c, kt, kit000, pahu, pahv, ptb, ptb, zlap, kjpt, 1);
  if (s) return s;
  cudaError_t e = launch_lbc<T>(zlap, c->jpi, c->jpj, (long)c->jpk * kjpt * c->nmem, 0, T(0), c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "tra_ldf_blp lbc");
  const bool zps = c->nam.ln_zps;
  if (zps) {  // GRADh of the first laplacian at the partial steps
    e = launch_zps_hde<T>(dom_now<T>(c), zlap, zglu, zglv, kjpt, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "tra_ldf_blp zps_hde");
  }
  if (kldf == 22) return run_ldf_triad<T>(c, kt, kit000, pahu, pahv, zlap, ptb, pta, kjpt, 2);
  return kldf == 20 ? run_ldf_lap<T>(c, pahu, pahv, zps ? zglu : nullptr, zps ? zglv : nullptr, zlap, pta, kjpt, 2)
                    : run_ldf_iso<T>(c, kt, kit000, pahu, pahv, zps ? zglu : nullptr, zps ? zglv : nullptr, zlap, ptb,
                                     pta, kjpt, 2);
}

template <class T>
int run_zdf(nemo_ctx* c, double p2dt, const void* ptb, void* pta, int kjpt, int is_trc, int clamp) {
  const nemo_namelist& nm = c->nam;
  ZdfArgs<T> a{};
  a.p2dt = (T)p2dt; a.ptb = (const T*)ptb; a.pta = (T*)pta; a.kjpt = kjpt;
  a.avt = (const T*)c->f[NEMO_F_AVT]; a.avs = (const T*)c->f[NEMO_F_AVS];
  a.ddm = nm.ln_zdfddm; a.is_trc = is_trc; a.clamp_sal = clamp;
  if (!is_trc && !a.avt) return fail(c, NEMO_ERR_UNBOUND, "tra_zdf_imp: avt must be bound");
  if ((is_trc || nm.ln_zdfddm) && !a.avs) return fail(c, NEMO_ERR_UNBOUND, "tra_zdf_imp: avs must be bound");
  if (nm.ln_traldf_iso || nm.ln_traldf_triad) {  // l_ldfslp (ldftra.F90:253-255)
    a.add = (const T*)c->f[nm.ln_traldf_msc ? NEMO_F_AKZ : NEMO_F_AH_WSLP2];
    if (!a.add) return fail(c, NEMO_ERR_UNBOUND, "tra_zdf_imp: ah_wslp2/akz must be bound with iso-neutral mixing");
  }
  cudaError_t e = launch_zdf<T>(dom_now<T>(c), a, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "tra_zdf_imp launch");
  return NEMO_OK;
}

template <class T>
int run_spg(nemo_ctx* c, int kt) {
  const nemo_namelist& nm = c->nam;
  void* const* F = c->f;
  const int need[] = {NEMO_F_UA, NEMO_F_VA, NEMO_F_UN, NEMO_F_VN, NEMO_F_SSHN, NEMO_F_SSHA, NEMO_F_UN_B,
                      NEMO_F_VN_B, NEMO_F_UB_B, NEMO_F_VB_B, NEMO_F_UA_B, NEMO_F_VA_B, NEMO_F_UN_ADV,
                      NEMO_F_VN_ADV, NEMO_F_UB2_B, NEMO_F_VB2_B, NEMO_F_UN_BF, NEMO_F_VN_BF, NEMO_F_UTAU,
                      NEMO_F_VTAU, NEMO_F_EMP, NEMO_F_RCDU_BOT};
  for (int id : need)
    if (!F[id]) return fail(c, NEMO_ERR_UNBOUND, "dyn_spg_ts: field %d must be bound", id);
  if (!nm.ln_bt_fw)
    for (int id : {NEMO_F_UB, NEMO_F_VB, NEMO_F_SSHB, NEMO_F_UTAU_B, NEMO_F_VTAU_B, NEMO_F_EMP_B})
      if (!F[id]) return fail(c, NEMO_ERR_UNBOUND, "dyn_spg_ts (ln_bt_fw=F): field %d must be bound", id);
  if (nm.ln_apr_dyn && (!F[NEMO_F_SSH_IB] || (!nm.ln_bt_fw && !F[NEMO_F_SSH_IBB])))
    return fail(c, NEMO_ERR_UNBOUND, "dyn_spg_ts (ln_apr_dyn): ssh_ib must be bound");
  const int vvl = !nm.ln_linssh, flux = vvl && !nm.ln_dynadv_vec;
  const int sc = nm.nvor_scheme;
  if (vvl) {
    for (int id : {NEMO_F_HT_N, NEMO_F_HU_N, NEMO_F_HV_N, NEMO_F_R1_HU_N, NEMO_F_R1_HV_N})
      if (!F[id]) return fail(c, NEMO_ERR_UNBOUND, "dyn_spg_ts (ln_linssh=F): depth field %d must be bound", id);
    if ((sc == NEMO_VOR_ENE || sc == NEMO_VOR_ENS || sc == NEMO_VOR_MIX) && !F[NEMO_F_E3F_N])
      return fail(c, NEMO_ERR_UNBOUND, "dyn_spg_ts (ln_linssh=F): e3f_n must be bound");
    if ((!nm.ln_bt_fw || flux) && (!F[NEMO_F_HU_B] || !F[NEMO_F_HV_B]))
      return fail(c, NEMO_ERR_UNBOUND, "dyn_spg_ts (ln_linssh=F): hu_b, hv_b must be bound");
    if (!nm.ln_bt_fw && (!F[NEMO_F_R1_HU_B] || !F[NEMO_F_R1_HV_B]))
      return fail(c, NEMO_ERR_UNBOUND, "dyn_spg_ts (ln_linssh=F, ln_bt_fw=F): r1_hu_b, r1_hv_b must be bound");
  }
  // kt-dependent scalars (:185-216, :346-349)
  const double z2dt_bf = (kt == nm.nit000 && nm.neuler == 0) ? nm.rn_rdt : 2.0 * nm.rn_rdt;
  int ll_init = nm.ln_bt_av;
  bool reweight = false;
  int ll_fw_start = 0;
  if (kt == nm.nit000) {
    if (nm.neuler == 0) ll_init = 1;
    ll_fw_start = (nm.ln_bt_fw || nm.neuler == 0) ? 1 : 0;
    reweight = true;
  }
  if (!nm.ln_bt_fw && nm.neuler == 0 && kt == nm.nit000 + 1) { ll_fw_start = 0; reweight = true; }
  if (reweight) {
    int jpit = 0;
    ts_wgt(c, nm.ln_bt_av, ll_fw_start, &jpit);
    c->icycle = jpit;
    CK(cudaMemcpyAsync(c->d_wgt1, c->wgt1.data(), c->wgt1.size() * 8, cudaMemcpyHostToDevice, c->stream), "weights");
    CK(cudaMemcpyAsync(c->d_wgt2, c->wgt2.data(), c->wgt2.size() * 8, cudaMemcpyHostToDevice, c->stream), "weights");
    float_weights(c);
    CK(cudaMemcpyAsync(c->d_wgtf, c->wgtf.data(), c->wgtf.size() * 4, cudaMemcpyHostToDevice, c->stream), "weights");
    CK(cudaStreamSynchronize(c->stream), "weights");
  }
  SpgArgs<T> a{};
  a.ua = (T*)F[NEMO_F_UA]; a.va = (T*)F[NEMO_F_VA]; a.un = (T*)F[NEMO_F_UN]; a.vn = (T*)F[NEMO_F_VN];
  a.ub = (const T*)F[NEMO_F_UB]; a.vb = (const T*)F[NEMO_F_VB];
  a.sshn = (const T*)F[NEMO_F_SSHN]; a.sshb = (const T*)F[NEMO_F_SSHB];
  a.un_b = (const T*)F[NEMO_F_UN_B]; a.vn_b = (const T*)F[NEMO_F_VN_B];
  a.ub_b = (const T*)F[NEMO_F_UB_B]; a.vb_b = (const T*)F[NEMO_F_VB_B];
  a.utau = (const T*)F[NEMO_F_UTAU]; a.vtau = (const T*)F[NEMO_F_VTAU];
  a.utau_b = (const T*)F[NEMO_F_UTAU_B]; a.vtau_b = (const T*)F[NEMO_F_VTAU_B];
  a.emp = (const T*)F[NEMO_F_EMP]; a.emp_b = (const T*)F[NEMO_F_EMP_B];
  a.rnf = (const T*)F[NEMO_F_RNF]; a.rnf_b = (const T*)F[NEMO_F_RNF_B];
  a.rCdU_bot = (const T*)F[NEMO_F_RCDU_BOT]; a.ssh_ib = (const T*)F[NEMO_F_SSH_IB]; a.ssh_ibb = (const T*)F[NEMO_F_SSH_IBB];
  a.ssha = (double*)F[NEMO_F_SSHA]; a.ua_b = (double*)F[NEMO_F_UA_B]; a.va_b = (double*)F[NEMO_F_VA_B];
  a.un_adv = (double*)F[NEMO_F_UN_ADV]; a.vn_adv = (double*)F[NEMO_F_VN_ADV];
  a.ub2_b = (double*)F[NEMO_F_UB2_B]; a.vb2_b = (double*)F[NEMO_F_VB2_B];
  a.un_bf = (double*)F[NEMO_F_UN_BF]; a.vn_bf = (double*)F[NEMO_F_VN_BF];
  a.zu_frc = (T*)c->spg_w[0]; a.zv_frc = (T*)c->spg_w[1]; a.zssh_frc = (T*)c->spg_w[2];
  a.zCdU_u = (T*)c->spg_w[3]; a.zCdU_v = (T*)c->spg_w[4];
  a.ring_ssh = (T*)c->ring[0]; a.ring_u = (T*)c->ring[1]; a.ring_v = (T*)c->ring[2];
  a.fx = (T*)c->spg_x[0]; a.fy = (T*)c->spg_x[1];
  a.du = (T*)c->spg_x[2]; a.dv = (T*)c->spg_x[3]; a.cu = (T*)c->spg_x[4]; a.cv = (T*)c->spg_x[5];
  a.zmu = (T*)c->spg_x[6]; a.zmv = (T*)c->spg_x[7];
  a.cache = c->p2_cache;
  a.hot = c->p2_hot;
  a.ff = c->spg_ff;
  a.wgt1 = c->d_wgt1; a.wgt2 = c->d_wgt2; a.wgtf = c->d_wgtf; a.nwgt = (int)c->wgt1.size();
  a.ln_bt_fw = nm.ln_bt_fw; a.ln_apr_dyn = nm.ln_apr_dyn; a.nvor = nm.nvor_scheme; a.ll_init = ll_init;
  a.icycle = c->icycle;
  // With time averaging every call restarts the barotropic levels, so the ring can
  // restart at slot 0; without it the levels carry over and the rotation continues.
  if (ll_init) c->ring0 = 0;
  a.ring0 = c->ring0;
  a.phase3_filter = !(kt == nm.nit000 && nm.neuler == 0);
  a.rdtbt = (T)c->rdtbt; a.grav = (T)nm.grav; a.r1_rau0 = (T)(1.0 / nm.rau0);
  a.scal_load = (T)nm.rn_scal_load; a.rn_bt_alpha = (T)nm.rn_bt_alpha;
  a.rn_atfp = nm.rn_atfp; a.r1_2dt_b = 1.0 / z2dt_bf;
  // depths and Coriolis factors: the domain's rest state, or the bound fields and
  // the per-member factors of this step with a variable volume
  const Dom<T> dn = dom_now<T>(c);
  a.vvl = vvl; a.flux = flux; a.een_e3f = nm.nn_een_e3f; a.sco = nm.ln_sco;
  a.hs = vvl ? c->n2 : 0;
  a.ht_n = dn.ht_0; a.hu_n = dn.hu_0; a.hv_n = dn.hv_0; a.r1_hu_n = dn.r1_hu_0; a.r1_hv_n = dn.r1_hv_0;
  a.hu_b = dn.hu_0; a.hv_b = dn.hv_0; a.r1_hu_b = dn.r1_hu_0; a.r1_hv_b = dn.r1_hv_0;
  a.zwz = dn.zwz; a.ftne = dn.ftne; a.ftnw = dn.ftnw; a.ftse = dn.ftse; a.ftsw = dn.ftsw;
  if (vvl) {
    auto ro = [&](int id) { return RO<T>((const T*)F[id]); };
    a.ht_n = ro(NEMO_F_HT_N); a.hu_n = ro(NEMO_F_HU_N); a.hv_n = ro(NEMO_F_HV_N);
    a.r1_hu_n = ro(NEMO_F_R1_HU_N); a.r1_hv_n = ro(NEMO_F_R1_HV_N);
    a.hu_b = ro(NEMO_F_HU_B); a.hv_b = ro(NEMO_F_HV_B); a.r1_hu_b = ro(NEMO_F_R1_HU_B); a.r1_hv_b = ro(NEMO_F_R1_HV_B);
    a.e3f_n = ro(NEMO_F_E3F_N);
    for (int w = 0; w < 5; ++w) a.cor_w[w] = (T*)c->spg_cor[w];
    a.zwz = (const T*)c->spg_cor[0]; a.ftne = (const T*)c->spg_cor[1]; a.ftnw = (const T*)c->spg_cor[2];
    a.ftse = (const T*)c->spg_cor[3]; a.ftsw = (const T*)c->spg_cor[4];
  }
  GridBar bar{c->bar_mem, c->bar_mem + 1, c->err_flag, (unsigned)(c->p2_blocks + c->bar_extra), c->bar_spins};
  cudaError_t e = launch_spg<T>(dn, a, bar, c->p2_blocks, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "dyn_spg_ts launch");
  c->ring0 = (c->ring0 + 3 * c->icycle) & 3;
  return NEMO_OK;
}

template <class T>
int run_ldf_slp(nemo_ctx* c, const void* prd, const void* pn2) {
  const nemo_namelist& nm = c->nam;
  const size_t n3 = (size_t)c->n3 * c->nmem, n2 = (size_t)c->n2 * c->nmem;
  if (!c->slp_w && cudaMalloc(&c->slp_w, (4 * n3 + 6 * n2) * sizeof(T)) != cudaSuccess)
    return fail(c, NEMO_ERR_NOMEM, "ldf_slp work arrays");
  T* w = (T*)c->slp_w;
  SlpArgs<T> a{};
  a.prd = (const T*)prd; a.pn2 = (const T*)pn2;
  a.gdept = (const T*)c->f[NEMO_F_GDEPT_N]; a.gdepw = (const T*)c->f[NEMO_F_GDEPW_N];
  a.nmln = (const int*)c->f[NEMO_F_NMLN];
  a.hmlp = (const T*)c->f[NEMO_F_HMLP]; a.hmlpt = (const T*)c->f[NEMO_F_HMLPT];
  a.uslp = (T*)c->f[NEMO_F_USLP]; a.vslp = (T*)c->f[NEMO_F_VSLP];
  a.wslpi = (T*)c->f[NEMO_F_WSLPI]; a.wslpj = (T*)c->f[NEMO_F_WSLPJ];
  if (nm.ln_zps) {
    if (!c->f[NEMO_F_GRU] || !c->f[NEMO_F_GRV])
      return fail(c, NEMO_ERR_UNBOUND, "ldf_slp with partial steps: gru and grv (zps_hde) must be bound");
    a.gru_b = (const T*)c->f[NEMO_F_GRU]; a.grv_b = (const T*)c->f[NEMO_F_GRV];
  }
  a.zu = w; a.zv = w + n3; a.zwi = w + 2 * n3; a.zwj = w + 3 * n3;
  T* w2 = w + 4 * n3;
  a.uml = w2; a.vml = w2 + n2; a.wiml = w2 + 2 * n2; a.wjml = w2 + 3 * n2; a.hu = w2 + 4 * n2; a.hv = w2 + 5 * n2;
  a.zeps = (T)1.e-20; a.zm1_g = (T)(-1.0 / nm.grav); a.zm1_2g = (T)(-0.5 / nm.grav);
  a.z1_slpmax = (T)(1.0 / (nm.rn_slpmax > 0 ? nm.rn_slpmax : 0.01));
  cudaError_t e = launch_ldf_slp<T>(dom_now<T>(c), a, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "ldf_slp launch");
  return NEMO_OK;
}

// ------------------------------------------------- the rest of a model step
// usrdef_sbc (usrdef_sbc.F90:62-190): GYRE's analytic surface forcing
int usr_check(nemo_ctx* c) {
  for (int id : {NEMO_F_GPHIT, NEMO_F_GPHIU, NEMO_F_GPHIV, NEMO_F_TSB, NEMO_F_TSN, NEMO_F_QSR, NEMO_F_QNS,
                 NEMO_F_EMP, NEMO_F_SFX, NEMO_F_UTAU, NEMO_F_VTAU, NEMO_F_TAUM})
    if (!c->f[id]) return fail(c, NEMO_ERR_UNBOUND, "usrdef_sbc: field %d must be bound", id);
  return NEMO_OK;
}
// the scalars of step kt (year 1 of a 360-day calendar): the amplitude and the
// denominator of T*, 23.5 zcos_sais1, the seasonal factors of E-P south and north,
// ztaun, and whether sbc swaps the before fields (kt /= nit000)
void usr_scalars(const nemo_namelist& nm, int kt, double v[7]) {
  const double rpi = 3.141592653589793, zyydd = 360.0, rjjhh = 24.0;
  const double ztime = (double)kt * nm.rn_rdt / (60.0 * 60.0);
  const double ztimemax1 = ((5. * 30.) + 21.) * 24., ztimemin1 = ztimemax1 + rjjhh * zyydd / 2;
  const double ztimemax2 = ((6. * 30.) + 21.) * 24., ztimemin2 = ztimemax2 - rjjhh * zyydd / 2;
  const double zemp_S = 0.7, zemp_N = 0.8, zemp_sais = 0.1, zTstar = 28.3;
  const double zcos_sais1 = nemo_cos((ztime - ztimemax1) / (ztimemin1 - ztimemax1) * rpi);
  const double zcos_sais2 = nemo_cos((ztime - ztimemax2) / (ztimemax2 - ztimemin2) * rpi);
  v[0] = zTstar * (1. + 1. / 50. * zcos_sais2);
  v[1] = 53.5 * (1 + 11 / 53.5 * zcos_sais2) * 2.;
  v[2] = 23.5 * zcos_sais1;
  v[3] = 1 - zemp_sais / zemp_S * zcos_sais1;
  v[4] = 1 - zemp_sais / zemp_N * zcos_sais1;
  const double ztimemax = ((5. * 30.) + 21.) * 24., ztimemin = ztimemax + rjjhh * zyydd / 2;
  const double ztau = 0.105 / std::sqrt(2.), ztau_sais = 0.015;
  v[5] = ztau - ztau_sais * nemo_cos((ztime - ztimemax) / (ztimemin - ztimemax) * rpi);
  v[6] = kt != nm.nit000 ? 1.0 : 0.0;
}
// the step's scalars into device memory, ahead of the step (and of its graph)
int usr_put(nemo_ctx* c, int kt) {
  if (!c->usr_s && cudaMalloc(&c->usr_s, 8 * sizeof(double)) != cudaSuccess)
    return fail(c, NEMO_ERR_NOMEM, "usrdef_sbc scalars");
  double v[7];
  usr_scalars(c->nam, kt, v);
  cudaError_t e = launch_usr_put(c->usr_s, v, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "usrdef_sbc scalars launch");
  return NEMO_OK;
}
template <class T>
int run_usrdef_sbc(nemo_ctx* c) {
  void* const* F = c->f;
  UsrSbcArgs<T> a{};
  a.gphit = (const T*)F[NEMO_F_GPHIT]; a.gphiu = (const T*)F[NEMO_F_GPHIU]; a.gphiv = (const T*)F[NEMO_F_GPHIV];
  a.tsb = (const T*)F[NEMO_F_TSB]; a.tsn = (const T*)F[NEMO_F_TSN];
  a.qsr = (T*)F[NEMO_F_QSR]; a.qns = (T*)F[NEMO_F_QNS]; a.emp = (T*)F[NEMO_F_EMP]; a.sfx = (T*)F[NEMO_F_SFX];
  a.utau = (T*)F[NEMO_F_UTAU]; a.vtau = (T*)F[NEMO_F_VTAU]; a.taum = (T*)F[NEMO_F_TAUM];
  a.utau_b = (T*)F[NEMO_F_UTAU_B]; a.vtau_b = (T*)F[NEMO_F_VTAU_B]; a.emp_b = (T*)F[NEMO_F_EMP_B];
  a.s = c->usr_s; a.gsum = c->gs_out;
  a.zsurf = c->usr_zsurf;
  a.rcp = c->nam.rcp > 0 ? c->nam.rcp : 3991.86795711963;
  const Dom<T> d = dom<T>(c);
  CK(launch_usr_sbc_a<T>(d, a, c->stream), "usrdef_sbc launch");
  CK(launch_globsum<T>((const T*)F[NEMO_F_EMP], d.tmask_i.p, c->n2, 1, c->nmem, c->gs_part, c->gs_nblk,
                       c->gs_out, c->stream),
     "usrdef_sbc glob_sum");
  CK(launch_usr_sbc_b<T>(d, a, c->stream), "usrdef_sbc launch");
  return NEMO_OK;
}

int model_fields(nemo_ctx* c, const char* what) {
  const nemo_namelist& nm = c->nam;
  if (nm.ln_usr)
    if (int s = usr_check(c)) return s;
  for (int id : {NEMO_F_UN, NEMO_F_VN, NEMO_F_WN, NEMO_F_UA, NEMO_F_VA, NEMO_F_UB, NEMO_F_VB, NEMO_F_UN_B,
                 NEMO_F_VN_B, NEMO_F_UB_B, NEMO_F_VB_B, NEMO_F_UA_B, NEMO_F_VA_B, NEMO_F_SSHB, NEMO_F_SSHN,
                 NEMO_F_SSHA, NEMO_F_TSB, NEMO_F_TSN, NEMO_F_TSA})
    if (!c->f[id]) return fail(c, NEMO_ERR_UNBOUND, "%s: field %d must be bound", what, id);
  if (!nm.ln_linssh || !nm.ln_bt_fw)
    return fail(c, NEMO_ERR_UNSUPPORTED, "%s: the linear free surface with ln_bt_fw only", what);
  return NEMO_OK;
}

template <class T>
int run_wzv(nemo_ctx* c, int kt) {
  const nemo_namelist& nm = c->nam;
  const double z1_2dt = (nm.neuler == 0 && kt == nm.nit000) ? 1.0 / nm.rn_rdt : 1.0 / (2.0 * nm.rn_rdt);
  cudaError_t e = launch_wzv<T>(dom_now<T>(c), (const T*)c->f[NEMO_F_UN], (const T*)c->f[NEMO_F_VN],
                                (T*)c->f[NEMO_F_WN], (T)z1_2dt, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "wzv launch");
  return NEMO_OK;
}

// dyn_zdf: the time step alone, or with the implicit vertical viscosity where the
// ocean avm is bound
int dyn_zdf_check(nemo_ctx* c) {
  void* const* F = c->f;
  for (int id : {NEMO_F_UA, NEMO_F_VA, NEMO_F_UB, NEMO_F_VB})
    if (!F[id]) return fail(c, NEMO_ERR_UNBOUND, "dyn_zdf: ua, va, ub and vb must be bound");
  if (!c->nam.ln_linssh && !c->nam.ln_dynadv_vec)
    for (int id : {NEMO_F_E3U_B, NEMO_F_E3V_B, NEMO_F_E3U_N, NEMO_F_E3V_N, NEMO_F_E3U_A, NEMO_F_E3V_A})
      if (!F[id]) return fail(c, NEMO_ERR_UNBOUND, "dyn_zdf (flux form, variable volume): e3u/e3v _b, _n, _a must be bound");
  if (!F[NEMO_F_AVM]) return NEMO_OK;
  for (int id : {NEMO_F_UA_B, NEMO_F_VA_B, NEMO_F_RCDU_BOT, NEMO_F_UTAU, NEMO_F_VTAU})
    if (!F[id]) return fail(c, NEMO_ERR_UNBOUND, "dyn_zdf with avm: ua_b, va_b, rcdu_bot, utau, vtau must be bound");
  const nemo_namelist& nm = c->nam;
  if (!nm.ln_linssh || nm.ln_isfcav || nm.ln_zad_Aimp)
    return fail(c, NEMO_ERR_UNSUPPORTED, "dyn_zdf with avm: a linear free surface without cavities or ln_zad_Aimp");
  return NEMO_OK;
}

template <class T>
int run_dyn_zdf_step(nemo_ctx* c, int kt) {
  const nemo_namelist& nm = c->nam;
  void* const* F = c->f;
  const double r2dt = (nm.neuler == 0 && kt == nm.nit000) ? nm.rn_rdt : 2.0 * nm.rn_rdt;
  cudaError_t e;
  if (!F[NEMO_F_AVM]) {
    const bool flux = !nm.ln_linssh && !nm.ln_dynadv_vec;
    e = launch_dyn_zdf_step<T>(dom_now<T>(c), (const T*)F[NEMO_F_UB], (const T*)F[NEMO_F_VB], (T*)F[NEMO_F_UA],
                               (T*)F[NEMO_F_VA], (T)r2dt, flux ? (const T*)F[NEMO_F_E3U_B] : nullptr,
                               flux ? (const T*)F[NEMO_F_E3V_B] : nullptr, flux ? (const T*)F[NEMO_F_E3U_A] : nullptr,
                               flux ? (const T*)F[NEMO_F_E3V_A] : nullptr, c->stream);
  } else {
    const size_t n = (size_t)c->n3 * c->nmem;
    if (!c->zdyn_w && cudaMalloc(&c->zdyn_w, 2 * n * sizeof(T)) != cudaSuccess)
      return fail(c, NEMO_ERR_NOMEM, "dyn_zdf work arrays");
    DynZdfArgs<T> a{};
    a.ub = (const T*)F[NEMO_F_UB]; a.vb = (const T*)F[NEMO_F_VB]; a.avm = (const T*)F[NEMO_F_AVM];
    a.rcdu = (const T*)F[NEMO_F_RCDU_BOT]; a.utau = (const T*)F[NEMO_F_UTAU]; a.vtau = (const T*)F[NEMO_F_VTAU];
    a.utau_b = F[NEMO_F_UTAU_B] ? (const T*)F[NEMO_F_UTAU_B] : a.utau;
    a.vtau_b = F[NEMO_F_VTAU_B] ? (const T*)F[NEMO_F_VTAU_B] : a.vtau;
    a.ua_b = (const double*)F[NEMO_F_UA_B]; a.va_b = (const double*)F[NEMO_F_VA_B];
    a.ua = (T*)F[NEMO_F_UA]; a.va = (T*)F[NEMO_F_VA];
    a.zwd = (T*)c->zdyn_w; a.zws = a.zwd + n;
    a.r2dt = (T)r2dt; a.zdt = (T)(r2dt * 0.5); a.rau0 = (T)nm.rau0;
    e = launch_dyn_zdf_imp<T>(dom_now<T>(c), a, c->stream);
  }
  if (e != cudaSuccess) return cuda_fail(c, e, "dyn_zdf launch");
  return NEMO_OK;
}

template <class T>
int run_tra_nxt(nemo_ctx* c, int kt) {
  const nemo_namelist& nm = c->nam;
  cudaError_t e = launch_tra_nxt<T>(dom<T>(c), (T*)c->f[NEMO_F_TSB], (T*)c->f[NEMO_F_TSN], (T*)c->f[NEMO_F_TSA],
                                    (T)nm.rn_atfp, nm.neuler == 0 && kt == nm.nit000, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "tra_nxt launch");
  return NEMO_OK;
}

template <class T>
int run_dyn_nxt(nemo_ctx* c, int kt) {
  const nemo_namelist& nm = c->nam;
  void* const* F = c->f;
  NxtArgs<T, double> a{};
  a.ua = (T*)F[NEMO_F_UA]; a.va = (T*)F[NEMO_F_VA]; a.un = (T*)F[NEMO_F_UN]; a.vn = (T*)F[NEMO_F_VN];
  a.ub = (T*)F[NEMO_F_UB]; a.vb = (T*)F[NEMO_F_VB];
  a.un_b = (T*)F[NEMO_F_UN_B]; a.vn_b = (T*)F[NEMO_F_VN_B]; a.ub_b = (T*)F[NEMO_F_UB_B]; a.vb_b = (T*)F[NEMO_F_VB_B];
  a.ua_b = (const double*)F[NEMO_F_UA_B]; a.va_b = (const double*)F[NEMO_F_VA_B];
  a.atfp = (T)nm.rn_atfp;
  a.euler = nm.neuler == 0 && kt == nm.nit000;
  cudaError_t e = launch_dyn_nxt<T>(dom<T>(c), a, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "dyn_nxt launch");
  return NEMO_OK;
}

template <class T>
int run_ssh_swp(nemo_ctx* c, int kt) {
  const nemo_namelist& nm = c->nam;
  cudaError_t e = launch_ssh_swp<T>(dom<T>(c), (T*)c->f[NEMO_F_SSHB], (T*)c->f[NEMO_F_SSHN],
                                    (const double*)c->f[NEMO_F_SSHA], (T)nm.rn_atfp,
                                    nm.neuler == 0 && kt == nm.nit000, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "ssh_swp launch");
  return NEMO_OK;
}

// ------------------------------------------------------------ z* time stepping
// The arguments of the k_vvl.cuh kernels from the bound fields (null where unbound).
template <class T>
VvlArgs<T> vvl_args(nemo_ctx* c, int kt) {
  const nemo_namelist& nm = c->nam;
  void* const* F = c->f;
  auto t = [&](int id) { return (T*)F[id]; };
  VvlArgs<T> a{};
  a.ssha = (const double*)F[NEMO_F_SSHA]; a.sshb = t(NEMO_F_SSHB); a.sshn = t(NEMO_F_SSHN);
  a.emp = t(NEMO_F_EMP); a.emp_b = t(NEMO_F_EMP_B); a.rnf = t(NEMO_F_RNF); a.rnf_b = t(NEMO_F_RNF_B);
  a.e3t_b = t(NEMO_F_E3T_B); a.e3t_n = t(NEMO_F_E3T_N); a.e3t_a = t(NEMO_F_E3T_A);
  a.e3u_n = t(NEMO_F_E3U_N); a.e3v_n = t(NEMO_F_E3V_N); a.e3u_a = t(NEMO_F_E3U_A); a.e3v_a = t(NEMO_F_E3V_A);
  a.e3u_b = t(NEMO_F_E3U_B); a.e3v_b = t(NEMO_F_E3V_B);
  a.e3w_n = t(NEMO_F_E3W_N); a.e3f_n = t(NEMO_F_E3F_N); a.e3w_b = t(NEMO_F_E3W_B);
  a.e3uw_n = t(NEMO_F_E3UW_N); a.e3vw_n = t(NEMO_F_E3VW_N); a.e3uw_b = t(NEMO_F_E3UW_B); a.e3vw_b = t(NEMO_F_E3VW_B);
  a.e3uw_0 = t(NEMO_F_E3UW_0); a.e3vw_0 = t(NEMO_F_E3VW_0);
  a.hu_a = t(NEMO_F_HU_A); a.hv_a = t(NEMO_F_HV_A); a.r1_hu_a = t(NEMO_F_R1_HU_A); a.r1_hv_a = t(NEMO_F_R1_HV_A);
  a.hu_n = t(NEMO_F_HU_N); a.hv_n = t(NEMO_F_HV_N); a.r1_hu_n = t(NEMO_F_R1_HU_N); a.r1_hv_n = t(NEMO_F_R1_HV_N);
  a.ht_n = t(NEMO_F_HT_N);
  a.hu_b = t(NEMO_F_HU_B); a.hv_b = t(NEMO_F_HV_B); a.r1_hu_b = t(NEMO_F_R1_HU_B); a.r1_hv_b = t(NEMO_F_R1_HV_B);
  a.gdept_n = t(NEMO_F_GDEPT_N); a.gdepw_n = t(NEMO_F_GDEPW_N); a.gde3w_n = t(NEMO_F_GDE3W_N);
  a.gdept_b = t(NEMO_F_GDEPT_B); a.gdepw_b = t(NEMO_F_GDEPW_B);
  a.ua = t(NEMO_F_UA); a.va = t(NEMO_F_VA); a.un = t(NEMO_F_UN); a.vn = t(NEMO_F_VN);
  a.ub = t(NEMO_F_UB); a.vb = t(NEMO_F_VB);
  a.un_b = t(NEMO_F_UN_B); a.vn_b = t(NEMO_F_VN_B); a.ub_b = t(NEMO_F_UB_B); a.vb_b = t(NEMO_F_VB_B);
  a.ua_b = (const double*)F[NEMO_F_UA_B]; a.va_b = (const double*)F[NEMO_F_VA_B];
  a.tsb = t(NEMO_F_TSB); a.tsn = t(NEMO_F_TSN); a.tsa = t(NEMO_F_TSA);
  a.tsc = t(NEMO_F_SBC_TSC); a.tsc_b = t(NEMO_F_SBC_TSC_B); a.qsr_hc = t(NEMO_F_QSR_HC); a.qsr_hc_b = t(NEMO_F_QSR_HC_B);
  a.atfp = (T)nm.rn_atfp;
  const double zfact1 = nm.rn_atfp * nm.rn_rdt;   // tranxt.F90:294-295, dynnxt.F90:223, sshwzv.F90:255
  a.zfact1 = (T)zfact1;
  a.zfact2 = (T)(zfact1 * (1.0 / nm.rau0));
  a.euler = nm.neuler == 0 && kt == nm.nit000;
  a.vec = nm.ln_dynadv_vec;
  a.traqsr = nm.ln_traqsr;
  a.nksr = c->nksr;
  return a;
}

enum { VVL_SF_NXT, VVL_SF_SWP, VVL_TRA_NXT, VVL_DYN_NXT, VVL_SSH_SWP };

template <class T>
int run_vvl(nemo_ctx* c, int kt, int what) {
  const VvlArgs<T> a = vvl_args<T>(c, kt);
  const Dom<T>& d0 = dom<T>(c);  // the rest-state scale factors
  cudaError_t e = cudaSuccess;
  switch (what) {
    case VVL_SF_NXT: e = launch_vvl_sf_nxt<T>(d0, a, c->stream); break;
    case VVL_SF_SWP: e = launch_vvl_sf_swp<T>(d0, a, c->stream); break;
    case VVL_TRA_NXT: e = launch_tra_nxt_vvl<T>(d0, a, c->stream); break;
    case VVL_DYN_NXT: e = launch_dyn_nxt_vvl<T>(d0, a, c->stream); break;
    default: e = launch_ssh_swp_vvl<T>(d0, a, (T*)c->f[NEMO_F_SSHB], (T*)c->f[NEMO_F_SSHN], c->stream); break;
  }
  if (e != cudaSuccess) return cuda_fail(c, e, "z* time-stepping launch");
  return NEMO_OK;
}

// the fields a z* routine reads or writes, and the pairs bound together
int vvl_check(nemo_ctx* c, const char* what, std::initializer_list<int> ids) {
  if (c->nam.ln_linssh) return fail(c, NEMO_ERR_ARG, "%s: variable volume only (ln_linssh = 0)", what);
  for (int id : ids)
    if (!c->f[id]) return fail(c, NEMO_ERR_UNBOUND, "%s: field %d must be bound", what, id);
  if (!c->f[NEMO_F_RNF] != !c->f[NEMO_F_RNF_B]) return fail(c, NEMO_ERR_UNBOUND, "%s: bind both rnf and rnf_b", what);
  return NEMO_OK;
}

// first-step mode of the forcing swaps: 0 swap, 1 Euler start (before = 0), 2 restart
int sbc_mode(const nemo_ctx* c, int kt) {
  if (kt != c->nam.nit000) return 0;
  return c->nam.neuler == 0 ? 1 : 2;
}
double rcp_of(const nemo_namelist& nm) { return nm.rcp > 0 ? nm.rcp : 3991.86795711963; }

template <class T>
int run_tra_sbc(nemo_ctx* c, int kt) {
  const nemo_namelist& nm = c->nam;
  void* const* F = c->f;
  SbcArgs<T> a{};
  a.qns = (T*)F[NEMO_F_QNS]; a.qsr = (T*)F[NEMO_F_QSR];
  a.emp = (const T*)F[NEMO_F_EMP]; a.sfx = (const T*)F[NEMO_F_SFX]; a.tsn = (const T*)F[NEMO_F_TSN];
  a.tsc = (T*)F[NEMO_F_SBC_TSC]; a.tsc_b = (T*)F[NEMO_F_SBC_TSC_B]; a.tsa = (T*)F[NEMO_F_TSA];
  const double rau0_rcp = nm.rau0 * rcp_of(nm);
  a.r1_rau0 = (T)(1.0 / nm.rau0); a.r1_rau0_rcp = (T)(1.0 / rau0_rcp);
  a.mode = sbc_mode(c, kt);
  a.zfact = (T)(a.mode == 1 ? 1.0 : 0.5);
  a.traqsr = nm.ln_traqsr; a.linssh = nm.ln_linssh;
  cudaError_t e = launch_tra_sbc<T>(dom_now<T>(c), a, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "tra_sbc launch");
  return NEMO_OK;
}

template <class T>
int run_tra_qsr(nemo_ctx* c, int kt) {
  const nemo_namelist& nm = c->nam;
  void* const* F = c->f;
  QsrArgs<T> a{};
  a.qsr = (const T*)F[NEMO_F_QSR]; a.gdepw = (const T*)F[NEMO_F_GDEPW_N];
  a.hc = (T*)F[NEMO_F_QSR_HC]; a.hc_b = (T*)F[NEMO_F_QSR_HC_B]; a.fraq = (T*)F[NEMO_F_FRAQSR_1LEV];
  a.tsa = (T*)F[NEMO_F_TSA];
  const double r1_rau0_rcp = 1.0 / (nm.rau0 * rcp_of(nm));
  a.zz0 = (T)(nm.rn_abs * r1_rau0_rcp); a.zz1 = (T)((1. - nm.rn_abs) * r1_rau0_rcp);
  a.xsi0r = (T)(1.0 / nm.rn_si0); a.xsi1r = (T)(1.0 / nm.rn_si1);
  a.r1_rau0_rcp = (T)r1_rau0_rcp;
  a.mode = sbc_mode(c, kt);
  a.z1_2 = (T)(a.mode == 1 ? 1.0 : 0.5);
  a.nksr = c->nksr;
  cudaError_t e = launch_tra_qsr<T>(dom_now<T>(c), a, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "tra_qsr launch");
  return NEMO_OK;
}

template <class T>
int run_zdf_mxl(nemo_ctx* c) {
  void* const* F = c->f;
  MxlArgs<T> a{};
  a.rn2b = (const T*)F[NEMO_F_RN2B]; a.avt = (const T*)F[NEMO_F_AVT];
  a.gdept = (const T*)F[NEMO_F_GDEPT_N]; a.gdepw = (const T*)F[NEMO_F_GDEPW_N];
  a.nmln = (int*)F[NEMO_F_NMLN]; a.hmlp = (T*)F[NEMO_F_HMLP]; a.hmlpt = (T*)F[NEMO_F_HMLPT];
  a.hmld = (T*)F[NEMO_F_HMLD];
  a.zn2_c = (T)(c->nam.grav * 0.01 * (1.0 / c->nam.rau0));
  a.avt_c = (T)5.e-4;
  a.nlb10 = c->nlb10;
  cudaError_t e = launch_zdf_mxl<T>(dom_now<T>(c), a, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "zdf_mxl launch");
  return NEMO_OK;
}

template <class T>
EosArgs<T> eos_args(const nemo_ctx* c, int what) {
  const nemo_namelist& nm = c->nam;
  EosArgs<T> a{};
  a.a0 = (T)nm.rn_a0; a.b0 = (T)nm.rn_b0; a.lambda1 = (T)nm.rn_lambda1; a.lambda2 = (T)nm.rn_lambda2;
  a.mu1 = (T)nm.rn_mu1; a.mu2 = (T)nm.rn_mu2; a.nu = (T)nm.rn_nu;
  a.rau0 = (T)nm.rau0; a.r1_rau0 = (T)(1.0 / nm.rau0); a.grav = (T)nm.grav;
  a.gdept = (const T*)c->f[NEMO_F_GDEPT_N]; a.gdepw = (const T*)c->f[NEMO_F_GDEPW_N];
  a.what = what;
  a.eos80 = nm.ln_eos80;
  a.e80_raw = c->e80_raw; a.e80_tay = c->e80_tay;
  a.e80_s0 = (float)c->e80_s0; a.e80_rho0 = (float)c->e80_rho0; a.e80_anom = (float)(c->e80_rho0 - nm.rau0);
  return a;
}

template <class T>
int run_eos(nemo_ctx* c, int what, const void* pts, void* prd, void* prhop, const void* pdep, void* pab,
            const void* pab_in, void* pn2) {
  EosArgs<T> a = eos_args<T>(c, what);
  a.pts = (const T*)pts; a.prd = (T*)prd; a.prhop = (T*)prhop; a.pdep = (const T*)pdep;
  a.pab = (T*)pab; a.pab_in = (const T*)pab_in; a.pn2 = (T*)pn2;
  cudaError_t e = launch_eos<T>(dom_now<T>(c), a, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "eos launch");
  return NEMO_OK;
}

template <class T>
int run_dyn_hpg(nemo_ctx* c) {
  cudaError_t e = launch_dyn_hpg<T>(dom_now<T>(c), (const T*)c->f[NEMO_F_RHD], (T*)c->f[NEMO_F_UA],
                                    (T*)c->f[NEMO_F_VA], (T)(-c->nam.grav * 0.5), c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "dyn_hpg launch");
  return NEMO_OK;
}

// the model step's eos + dyn_hpg: rhd, rhop and gdept_n bound, the simplified eos,
// z-coordinate with full steps
bool hpg_on(const nemo_ctx* c) {
  const nemo_namelist& nm = c->nam;
  return c->f[NEMO_F_RHD] && c->f[NEMO_F_RHOP] && c->f[NEMO_F_GDEPT_N] && (nm.ln_seos || nm.ln_eos80) &&
         !nm.ln_zps && !nm.ln_sco && !nm.ln_isfcav;
}

// the model step's iso-neutral slopes from the before tracers (step.F90:127-150):
// the simplified eos, rotated diffusion, z-coordinate with full steps, and every
// field of the chain bound
bool slopes_on(const nemo_ctx* c) {
  const nemo_namelist& nm = c->nam;
  if (!(nm.ln_seos || nm.ln_eos80) || !nm.ln_traldf_iso || nm.ln_zps || nm.ln_sco || nm.ln_isfcav) return false;
  for (int id : {NEMO_F_RN2B, NEMO_F_RHD, NEMO_F_GDEPT_N, NEMO_F_GDEPW_N, NEMO_F_NMLN, NEMO_F_HMLP, NEMO_F_HMLPT,
                 NEMO_F_USLP, NEMO_F_VSLP, NEMO_F_WSLPI, NEMO_F_WSLPJ, NEMO_F_AVT})
    if (!c->f[id]) return false;
  return true;
}

// eos_rab(tsb, rab_b), bn2(tsb, rab_b, rn2b), zdf_mxl, eos(tsb, rhd, gdept_0) and
// ldf_slp(rhd, rn2b) (step.F90:127-150). With the vertical physics on, rn2b is
// already formed (run_vphys) and only zdf_mxl onwards runs. gdept_0 is the bound
// gdept_n: the linear free surface keeps the rest-state depths.
template <class T>
int run_slopes(nemo_ctx* c, bool rn2b_done) {
  void* const* F = c->f;
  int s = NEMO_OK;
  if (!rn2b_done) {
    if (!c->rab_w && cudaMalloc(&c->rab_w, 2 * (size_t)c->n3 * c->nmem * sizeof(T)) != cudaSuccess)
      return fail(c, NEMO_ERR_NOMEM, "rab_b work array");
    s = run_eos<T>(c, 2, F[NEMO_F_TSB], nullptr, nullptr, nullptr, c->rab_w, nullptr, nullptr);
    if (!s) s = run_eos<T>(c, 3, F[NEMO_F_TSB], nullptr, nullptr, nullptr, nullptr, c->rab_w, F[NEMO_F_RN2B]);
  }
  if (!s) s = run_zdf_mxl<T>(c);
  if (!s) s = run_eos<T>(c, 0, F[NEMO_F_TSB], F[NEMO_F_RHD], nullptr, F[NEMO_F_GDEPT_N], nullptr, nullptr, nullptr);
  if (!s) s = run_ldf_slp<T>(c, F[NEMO_F_RHD], F[NEMO_F_RN2B]);
  return s;
}

// zdf_phy (zdfphy.F90:243-316) with the TKE closure: zdf_sh2, then the column
// kernel (tke_tke, tke_avn, the ocean Kz, zdf_evd, avs, the closed lbc_lnk)
bool zphy_bound(const nemo_ctx* c) {
  for (int id : {NEMO_F_UB, NEMO_F_VB, NEMO_F_UN, NEMO_F_VN, NEMO_F_AVM_K, NEMO_F_AVT_K, NEMO_F_AVM, NEMO_F_AVT,
                 NEMO_F_EN, NEMO_F_DISSL, NEMO_F_RN2, NEMO_F_RN2B, NEMO_F_TAUM, NEMO_F_GDEPW_N})
    if (!c->f[id]) return false;
  return true;
}
bool zphy_covered(const nemo_namelist& nm) {
  return nm.ln_zdftke && nm.nn_etau == 0 && !nm.ln_drg_tke && !nm.ln_isfcav && nm.ln_linssh && !nm.ln_sco;
}
int zphy_check(nemo_ctx* c) {
  if (!zphy_covered(c->nam))
    return fail(c, NEMO_ERR_UNSUPPORTED,
                "zdf_phy: the TKE closure with nn_etau = 0, ln_drg off, a linear free surface and z-levels");
  if (!zphy_bound(c))
    return fail(c, NEMO_ERR_UNBOUND,
                "zdf_phy: ub vb un vn avm_k avt_k avm avt en dissl rn2 rn2b taum gdepw_n must be bound");
  return NEMO_OK;
}

template <class T>
int run_zdf_phy(nemo_ctx* c) {
  const nemo_namelist& nm = c->nam;
  const size_t n = (size_t)c->n3 * c->nmem;
  if (!c->zphy_w && cudaMalloc(&c->zphy_w, 5 * n * sizeof(T)) != cudaSuccess)
    return fail(c, NEMO_ERR_NOMEM, "zdf_phy work arrays");
  void* const* F = c->f;
  ZphyArgs<T> a{};
  a.ub = (const T*)F[NEMO_F_UB]; a.vb = (const T*)F[NEMO_F_VB];
  a.un = (const T*)F[NEMO_F_UN]; a.vn = (const T*)F[NEMO_F_VN];
  a.rn2 = (const T*)F[NEMO_F_RN2]; a.rn2b = (const T*)F[NEMO_F_RN2B]; a.taum = (const T*)F[NEMO_F_TAUM];
  a.gdepw = (const T*)F[NEMO_F_GDEPW_N]; a.fr_i = (const T*)F[NEMO_F_FR_I];
  a.avm_k = (T*)F[NEMO_F_AVM_K]; a.avt_k = (T*)F[NEMO_F_AVT_K]; a.avm = (T*)F[NEMO_F_AVM];
  a.avt = (T*)F[NEMO_F_AVT]; a.avs = (T*)F[NEMO_F_AVS]; a.en = (T*)F[NEMO_F_EN]; a.dissl = (T*)F[NEMO_F_DISSL];
  T* w = (T*)c->zphy_w;
  a.sh2 = w; a.apdlr = w + n; a.zdiag = w + 2 * n; a.zd_up = w + 3 * n; a.zd_lw = w + 4 * n;
  // the constants of zdf_tke_init (zdftke.F90:663-690), tke_tke and tke_avn
  const double rdt = nm.rn_rdt, zrhoa = 1.22, zcdrag = 1.5e-3;
  const double rmxl_min = 1.e-6 / (nm.rn_ediff * std::sqrt(nm.rn_emin));
  a.rdt = (T)rdt; a.zbbrau = (T)(nm.rn_ebb / nm.rau0); a.zfact1 = (T)(-.5 * rdt);
  a.zfact2 = (T)(1.5 * rdt * nm.rn_ediss); a.zfact3 = (T)(0.5 * nm.rn_ediss);
  a.rn_emin = (T)nm.rn_emin; a.rn_emin0 = (T)nm.rn_emin0; a.rn_bshear = (T)nm.rn_bshear;
  a.rn_ediff = (T)nm.rn_ediff; a.rn_lc = (T)nm.rn_lc; a.rn_evd = (T)nm.rn_evd;
  a.rn_avm0 = (T)nm.rn_avm0; a.rn_avt0 = (T)nm.rn_avt0;
  a.ri_cri = (T)(2.0 / (2.0 + nm.rn_ediss / nm.rn_ediff)); a.rmxl_min = (T)rmxl_min;
  a.rn_mxl0 = (T)(nm.ln_mxl0 ? rmxl_min : nm.rn_mxl0);
  a.zraug = (T)(0.4 * 2.e5 / (nm.rau0 * nm.grav));
  a.rsmall = (T)(0.5 * 2.220446049250313e-16);
  a.lc_cof1 = (T)(0.5 * 0.016 * 0.016 / (zrhoa * zcdrag));
  a.lc_cof2 = (T)(0.016 / std::sqrt(zrhoa * zcdrag));
  a.rpi = (T)3.141592653589793;
  a.nn_pdl = nm.nn_pdl; a.nn_mxl = nm.nn_mxl; a.ln_mxl0 = nm.ln_mxl0; a.ln_lc = nm.ln_lc;
  a.ln_zdfevd = nm.ln_zdfevd; a.nn_evdm = nm.nn_evdm;
  cudaError_t e = launch_zdf_phy<T>(dom_now<T>(c), a, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "zdf_phy launch");
  return NEMO_OK;
}

// the momentum trends of the model step (step.F90:190-192): dyn_adv in the vector
// form (keg C2 + zad), dyn_vor with vor_ene of the total vorticity (the Coriolis
// term alone for linear dynamics, dynvor.F90:904-913), dyn_ldf where the viscosity
// ahmt, ahmf is bound
int mom_check(nemo_ctx* c) {
  const nemo_namelist& nm = c->nam;
  if (!nm.ln_dynadv_OFF && (!nm.ln_dynadv_vec || nm.nn_dynkeg != 0))
    return fail(c, NEMO_ERR_UNSUPPORTED, "stp_model: momentum advection in the vector form with nn_dynkeg = 0 only");
  if (nm.nvor_scheme != NEMO_VOR_ENE)
    return fail(c, NEMO_ERR_UNSUPPORTED, "stp_model: the energy-conserving vorticity scheme (ENE) only");
  if (nm.ln_sco) return fail(c, NEMO_ERR_UNSUPPORTED, "stp_model: z-coordinate only");
  if (c->f[NEMO_F_AHMT] && c->f[NEMO_F_AHMF] && !nm.ln_linssh)
    return fail(c, NEMO_ERR_UNSUPPORTED, "stp_model: the lateral viscosity of a linear free surface only");
  return NEMO_OK;
}
template <class T>
int run_mom_trends(nemo_ctx* c) {
  const nemo_namelist& nm = c->nam;
  void* const* F = c->f;
  const Dom<T> d = dom_now<T>(c);
  const T *un = (const T*)F[NEMO_F_UN], *vn = (const T*)F[NEMO_F_VN];
  T *ua = (T*)F[NEMO_F_UA], *va = (T*)F[NEMO_F_VA];
  if (!nm.ln_dynadv_OFF) {
    CK(launch_dyn_keg<T>(d, un, vn, ua, va, c->stream), "dyn_keg launch");
    CK(launch_dyn_zad<T>(d, un, vn, (const T*)F[NEMO_F_WN], ua, va, c->stream), "dyn_zad launch");
  }
  CK(launch_vor_ene<T>(d, nm.ln_dynadv_OFF ? 1 : 4, un, vn, ua, va, c->stream), "vor_ene launch");
  if (F[NEMO_F_AHMT] && F[NEMO_F_AHMF])
    CK(launch_dyn_ldf_lap<T>(d, (const T*)F[NEMO_F_AHMT], (const T*)F[NEMO_F_AHMF], (const T*)F[NEMO_F_UB],
                             (const T*)F[NEMO_F_VB], ua, va, T(1), c->stream),
       "dyn_ldf_lap launch");
  return NEMO_OK;
}

// the model step's vertical physics (step.F90:127-133): an equation of state, the
// TKE closure as zdf_phy covers it, z-levels with full steps, every field bound
bool zphy_on(const nemo_ctx* c) {
  const nemo_namelist& nm = c->nam;
  return zphy_covered(nm) && (nm.ln_seos || nm.ln_eos80) && !nm.ln_zps && zphy_bound(c) && c->f[NEMO_F_GDEPT_N];
}
// rab_3d and bn2 of the before and now tracers, then zdf_phy
template <class T>
int run_vphys(nemo_ctx* c) {
  void* const* F = c->f;
  const size_t b2 = 2 * (size_t)c->n3 * c->nmem * sizeof(T);
  if (!c->rab_w && cudaMalloc(&c->rab_w, b2) != cudaSuccess) return fail(c, NEMO_ERR_NOMEM, "rab_b work array");
  if (!c->rab_n && cudaMalloc(&c->rab_n, b2) != cudaSuccess) return fail(c, NEMO_ERR_NOMEM, "rab_n work array");
  int s = run_eos<T>(c, 2, F[NEMO_F_TSB], nullptr, nullptr, nullptr, c->rab_w, nullptr, nullptr);
  if (!s) s = run_eos<T>(c, 2, F[NEMO_F_TSN], nullptr, nullptr, nullptr, c->rab_n, nullptr, nullptr);
  if (!s) s = run_eos<T>(c, 3, F[NEMO_F_TSB], nullptr, nullptr, nullptr, nullptr, c->rab_w, F[NEMO_F_RN2B]);
  if (!s) s = run_eos<T>(c, 3, F[NEMO_F_TSN], nullptr, nullptr, nullptr, nullptr, c->rab_n, F[NEMO_F_RN2]);
  if (!s) s = run_zdf_phy<T>(c);
  return s;
}

bool sbc_bound(const nemo_ctx* c) {
  for (int id : {NEMO_F_QNS, NEMO_F_QSR, NEMO_F_EMP, NEMO_F_SFX, NEMO_F_SBC_TSC, NEMO_F_SBC_TSC_B})
    if (!c->f[id]) return false;
  return true;
}
bool qsr_bound(const nemo_ctx* c) {
  for (int id : {NEMO_F_QSR, NEMO_F_GDEPW_N, NEMO_F_QSR_HC, NEMO_F_QSR_HC_B, NEMO_F_FRAQSR_1LEV})
    if (!c->f[id]) return false;
  return true;
}

// stp_ctl and dia_hsb (k_diag.cuh)
template <class T>
int run_stp_ctl(nemo_ctx* c) {
  cudaError_t e = launch_stp_ctl<T>(dom<T>(c), (const T*)c->f[NEMO_F_SSHN], (const T*)c->f[NEMO_F_UN],
                                    (const T*)c->f[NEMO_F_TSN], c->ctl_part, c->ctl_nblk, c->someoce, c->ctl_out,
                                    c->ctl_idx, c->ctl_flag, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "stp_ctl launch");
  return NEMO_OK;
}

template <class T>
HsbArgs<T> hsb_args(nemo_ctx* c) {
  HsbArgs<T> a{};
  const size_t n2 = c->n2, n3 = c->n3, nm = c->nmem;
  a.tsn = (T*)c->f[NEMO_F_TSN]; a.tsb = (T*)c->f[NEMO_F_TSB];
  a.sshn = (const T*)c->f[NEMO_F_SSHN]; a.emp = (const T*)c->f[NEMO_F_EMP]; a.rnf = (const T*)c->f[NEMO_F_RNF];
  a.tsc = (const T*)c->f[NEMO_F_SBC_TSC]; a.qsr = (const T*)c->f[NEMO_F_QSR]; a.wn = (const T*)c->f[NEMO_F_WN];
  a.e3t = dom_now<T>(c).e3t_n;
  double* m = c->hsb_mem;
  a.surf = m; a.tmask_h = m + n2;
  a.ssh_ini = m + 2 * n2; a.ssh_hc_ini = a.ssh_ini + nm * n2; a.ssh_sc_ini = a.ssh_hc_ini + nm * n2;
  a.e3t_ini = a.ssh_sc_ini + nm * n2; a.hc_ini = a.e3t_ini + nm * n3; a.sc_ini = a.hc_ini + nm * n3;
  a.state = c->hsb_state; a.out = c->hsb_out;
  const double rcp = c->nam.rcp > 0 ? c->nam.rcp : 3991.86795711963;
  a.rdt = c->nam.rn_rdt; a.r1_rau0 = 1.0 / c->nam.rau0; a.r1_rau0_rcp = 1.0 / (c->nam.rau0 * rcp);
  a.linssh = c->nam.ln_linssh; a.traqsr = c->nam.ln_traqsr;
  return a;
}

int hsb_check(nemo_ctx* c) {
  if (!c->hsb_on) return fail(c, NEMO_ERR_STATE, "dia_hsb: call nemo_gpu_dia_hsb_init first");
  if (!c->f[NEMO_F_TSN] || !c->f[NEMO_F_TSB] || !c->f[NEMO_F_SSHN] || !c->f[NEMO_F_EMP] || !c->f[NEMO_F_SBC_TSC] ||
      !c->f[NEMO_F_WN] || (c->nam.ln_traqsr && !c->f[NEMO_F_QSR]))
    return fail(c, NEMO_ERR_UNBOUND, "dia_hsb: tsn, tsb, sshn, emp, sbc_tsc, wn (and qsr) must be bound");
  return NEMO_OK;
}

template <class T>
int run_dia_hsb(nemo_ctx* c) {
  cudaError_t e = launch_dia_hsb<T>(dom<T>(c), hsb_args<T>(c), c->hsb_part, c->hsb_nblk, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "dia_hsb launch");
  return NEMO_OK;
}

template <class T>
int run_hotpath(nemo_ctx* c, int kt, bool staged, bool model = false) {
  const nemo_namelist& nm = c->nam;
  void* const* F = c->f;
  if (!F[NEMO_F_TSB] || !F[NEMO_F_TSN] || !F[NEMO_F_TSA] || !F[NEMO_F_WN])
    return fail(c, NEMO_ERR_UNBOUND, "stp_hotpath: tsb, tsn, tsa, un, vn, wn must be bound");
  auto mark = [&](int i) { if (c->timing) cudaEventRecord(c->tev[i], c->stream); };
  // the kernel clock is installed for this thread until the function returns
  struct ClockGuard {
    explicit ClockGuard(KernelClock* k, const LaunchShape* sh) { t_kclock = k; t_shape = sh; }
    ~ClockGuard() { t_kclock = nullptr; t_shape = nullptr; }
  } guard(c->timing ? &c->kc : nullptr, &c->shape);
  if (c->timing) {
    c->kc.n = 0;
    cudaEventRecord(c->kc.ev[0], c->stream);
  }
  mark(0);
  if (model) {  // ua = va = 0 (step.F90:183-184)
    if (int s = dyn_zdf_check(c)) return s;
    if (nm.ln_usr)  // sbc (step.F90:116), its scalars put by stp_common
      if (int s = run_usrdef_sbc<T>(c)) return s;
    if (int s = mom_check(c)) return s;
    const bool vphys = zphy_on(c);
    if (vphys) {
      int s = run_vphys<T>(c);
      if (s) return s;
    }
    if (slopes_on(c)) {
      int s = run_slopes<T>(c, vphys);
      if (s) return s;
    }
    // ssh_nxt's div_hor and wzv (step.F90:156-160): the now vertical velocity of
    // dyn_adv (ssha comes from dyn_spg_ts with the split-explicit free surface)
    if (int s = run_wzv<T>(c, kt)) return s;
    const size_t bytes = (size_t)c->n3 * c->nmem * sizeof(T);
    CK(cudaMemsetAsync(F[NEMO_F_UA], 0, bytes, c->stream), "ua = 0");
    CK(cudaMemsetAsync(F[NEMO_F_VA], 0, bytes, c->stream), "va = 0");
    if (int s = run_mom_trends<T>(c)) return s;
    if (hpg_on(c)) {  // eos of tsn at gdept_n (step.F90:165) and dyn_hpg (:193)
      int s = run_eos<T>(c, 1, F[NEMO_F_TSN], F[NEMO_F_RHD], F[NEMO_F_RHOP], F[NEMO_F_GDEPT_N], nullptr, nullptr,
                         nullptr);
      if (!s) s = run_dyn_hpg<T>(c);
      if (s) return s;
    }
  }
  // Staged (host copies pending): each part waits only for the copies of the fields it
  // reads or writes -- dyn_spg_ts starts while the tracers and slopes still upload,
  // and the downloads of what it writes start when it ends (ev_spg_done).
  c->spg_done_valid = false;
  if (staged)  // the iso-neutral coefficients the first pass may zero on this stream
    if (wait_field(c, c->stream, NEMO_F_AH_WSLP2, true) || wait_field(c, c->stream, NEMO_F_AKZ, true))
      return NEMO_ERR_CUDA;
  const bool forced = model && sbc_bound(c);  // tra_sbc (and tra_qsr) before tra_adv
  const bool fused = nm.ln_traldf_iso && !nm.ln_traldf_blp && !c->no_fusion && !forced;
  LdfArgs<T> la{};
  // The iso-neutral fluxes read tsb and the slopes only, and dyn_spg_ts touches
  // neither them nor their outputs: outside per-kernel timing they run on the side
  // stream beside dyn_spg_ts and join before FCT stage c adds their divergence.
  const bool overlap = fused && !c->timing;
  if (fused) {
    int s = iso_args<T>(c, kt, nm.nit000, F[NEMO_F_AHTU], F[NEMO_F_AHTV], F[NEMO_F_GTSU], F[NEMO_F_GTSV],
                        F[NEMO_F_TSB], F[NEMO_F_TSB], F[NEMO_F_TSA], 2, 1, &la);
    if (s) return s;
    if (overlap) {
      CK(cudaEventRecord(c->ev_fork, c->stream), "fork");
      CK(cudaStreamWaitEvent(c->side, c->ev_fork, 0), "fork");
      if (staged)
        for (int id : {NEMO_F_TSB, NEMO_F_USLP, NEMO_F_VSLP, NEMO_F_WSLPI, NEMO_F_WSLPJ, NEMO_F_AHTU, NEMO_F_AHTV,
                       NEMO_F_GTSU, NEMO_F_GTSV, NEMO_F_E3U_N, NEMO_F_E3V_N, NEMO_F_E3W_N})
          if (wait_field(c, c->side, id, false)) return NEMO_ERR_CUDA;
      CK(launch_iso_flux<T>(dom_now<T>(c), la, c->side), "iso fluxes");
      CK(cudaEventRecord(c->ev_join, c->side), "join");
    }
  }
  if (staged)
    for (int id = 0; id < NEMO_F_COUNT; ++id)
      if (spg_reads(id) && wait_field(c, c->stream, id, spg_writes(id))) return NEMO_ERR_CUDA;
  int s = run_spg<T>(c, kt);
  if (s) return s;
  if (model) {  // div_hor + wzv after dyn_spg_ts (step.F90:206-211), the dyn_zdf time step
    if ((s = run_wzv<T>(c, kt))) return s;
    if ((s = run_dyn_zdf_step<T>(c, kt))) return s;
  }
  if (staged) {
    CK(cudaEventRecord(c->ev_spg_done, c->stream), "end of dyn_spg_ts");
    if (join_copies(c)) return NEMO_ERR_CUDA;  // the tracer part: every remaining copy
  }
  mark(1);
  if (forced) {  // step.F90:230-233
    CK(cudaMemsetAsync(F[NEMO_F_TSA], 0, 2 * (size_t)c->n3 * c->nmem * sizeof(T), c->stream), "tsa = 0");
    if ((s = run_tra_sbc<T>(c, kt))) return s;
    if (nm.ln_traqsr && (s = run_tra_qsr<T>(c, kt))) return s;
  }
  const double r2dt = (nm.neuler == 0 && kt == nm.nit000) ? nm.rn_rdt : 2.0 * nm.rn_rdt;
  const int fct_h = nm.nn_fct_h ? nm.nn_fct_h : 2, fct_v = nm.nn_fct_v ? nm.nn_fct_v : 2;  // &namtra_adv
  if (fused) {
    // tsa = 0, tra_adv and tra_ldf (iso-neutral, first pass): the iso-neutral
    // fluxes, then the three FCT stages; the last adds both the corrected
    // advective trend and the iso-neutral divergence of each point, in the
    // reference's order
    if (overlap) CK(cudaStreamWaitEvent(c->stream, c->ev_join, 0), "join");
    else CK(launch_iso_flux<T>(dom_now<T>(c), la, c->stream), "iso fluxes");
    mark(5);  // timed: the iso-neutral fluxes are tra_ldf's, the three FCT stages tra_adv's
    s = run_fct<T>(c, r2dt, F[NEMO_F_UN], F[NEMO_F_VN], F[NEMO_F_WN], 1, F[NEMO_F_TSB], F[NEMO_F_TSN], nullptr,
                   F[NEMO_F_TSA], 2, fct_h, fct_v, &la);
    if (s) return s;
    cudaError_t e = launch_iso_edges<T>(dom_now<T>(c), la, !nm.ln_traldf_msc, nm.ln_traldf_msc, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "iso edges");
    mark(2);
  } else {
  // tsa = 0 (step.F90:234) folded into the first trend (pta_in = NULL), or, with the
  // surface forcing of the model step, tsa = 0, tra_sbc, tra_qsr and FCT adding on
  s = run_fct<T>(c, r2dt, F[NEMO_F_UN], F[NEMO_F_VN], F[NEMO_F_WN], 1, F[NEMO_F_TSB], F[NEMO_F_TSN], forced ? F[NEMO_F_TSA] : nullptr,
                 F[NEMO_F_TSA], 2, fct_h, fct_v);
  if (s) return s;
  mark(2);
  if (nm.ln_traldf_blp)  // traldf.F90:75-76
    s = run_ldf_blp<T>(c, kt, nm.nit000, F[NEMO_F_AHTU], F[NEMO_F_AHTV], F[NEMO_F_GTSU], F[NEMO_F_GTSV],
                       F[NEMO_F_TSB], F[NEMO_F_TSA], 2, nm.ln_traldf_iso ? 21 : nm.ln_traldf_triad ? 22 : 20);
  else if (nm.ln_traldf_triad)  // np_lap_it (traldf.F90:73-74)
    s = run_ldf_triad<T>(c, kt, nm.nit000, F[NEMO_F_AHTU], F[NEMO_F_AHTV], F[NEMO_F_TSB], F[NEMO_F_TSB], F[NEMO_F_TSA],
                         2, 1);
  else if (nm.ln_traldf_iso)
    s = run_ldf_iso<T>(c, kt, nm.nit000, F[NEMO_F_AHTU], F[NEMO_F_AHTV], F[NEMO_F_GTSU], F[NEMO_F_GTSV], F[NEMO_F_TSB],
                       F[NEMO_F_TSB], F[NEMO_F_TSA], 2, 1);
  else
    s = run_ldf_lap<T>(c, F[NEMO_F_AHTU], F[NEMO_F_AHTV], F[NEMO_F_GTSU], F[NEMO_F_GTSV], F[NEMO_F_TSB], F[NEMO_F_TSA], 2, 1);
  if (s) return s;
  }
  mark(3);
  s = run_zdf<T>(c, r2dt, F[NEMO_F_TSB], F[NEMO_F_TSA], 2, 0, 1);
  if (s) return s;
  if (model) {  // tra_nxt, dyn_nxt, ssh_swp (step.F90:277-279), dia_hsb (:282), stp_ctl (:305)
    if ((s = run_tra_nxt<T>(c, kt))) return s;
    if ((s = run_dyn_nxt<T>(c, kt))) return s;
    if ((s = run_ssh_swp<T>(c, kt))) return s;
    if (c->hsb_on) {
      if ((s = hsb_check(c))) return s;
      if ((s = run_dia_hsb<T>(c))) return s;
    }
    if ((s = run_stp_ctl<T>(c))) return s;
  }
  if (c->timing) {
    mark(4);
    CK(cudaEventSynchronize(c->tev[4]), "timing");
    float rms[4] = {};
    for (int i = 0; i < 4; ++i) cudaEventElapsedTime(&rms[i], c->tev[i], c->tev[i + 1]);
    if (fused) {  // the fluxes ran first inside the tracer window
      float ldf = 0;
      cudaEventElapsedTime(&ldf, c->tev[1], c->tev[5]);
      rms[1] -= ldf;
      rms[2] += ldf;
    }
    for (int i = 0; i < 4; ++i) c->tms[i] += rms[i];
    c->tcalls += 1;
    for (int i = 0; i < c->kc.n; ++i) {
      float ms = 0;
      cudaEventElapsedTime(&ms, c->kc.ev[i], c->kc.ev[i + 1]);
      c->kms[c->kc.id[i]] += ms;
      c->kcnt[c->kc.id[i]] += 1;
    }
  }
  if (staged) c->spg_done_valid = true;
  return NEMO_OK;
}

}  // namespace

// ================================================================== C ABI
extern "C" {

// The EOS-80 tables on the device. FP32 evaluates each polynomial re-expanded in
// s' = zs - s0 about the reference salinity's s0 = sqrt((35 + 20) / 40), with the
// density's constant term (its value at 35 psu, 0 degC, 0 m) kept apart: in the
// monomial basis about zs = 0 the terms reach ~900 kg/m3 and cancel to the density,
// so FP32 would lose the density anomaly (~1e-4 kg/m3 against neighbour differences
// of 1e-3..1e-1); about s0 the terms are of the size of the anomaly itself. The
// re-expansion is exact in FP64 (binomial sums) and then rounded to FP32.
int upload_eos80(nemo_ctx* c) {
  static const double raw[3][4][7][7] = NEMO_EOS80_TABLE;
  const double s0 = std::sqrt((35.0 + NEMO_EOS80_RDELTAS) * NEMO_EOS80_R1_S0);
  std::vector<float> tay(3 * 4 * 49, 0.0f);
  double binom[7][7] = {};
  for (int n = 0; n < 7; ++n) {
    binom[n][0] = 1.0;
    for (int r = 1; r <= n; ++r) binom[n][r] = binom[n - 1][r - 1] + (r <= n - 1 ? binom[n - 1][r] : 0.0);
  }
  for (int t = 0; t < 3; ++t)
    for (int k = 0; k < 4; ++k)
      for (int j = 0; j < 7; ++j)
        for (int ip = 0; ip < 7; ++ip) {
          double v = 0.0;
          for (int i = ip; i < 7; ++i) v += raw[t][k][i][j] * binom[i][ip] * std::pow(s0, i - ip);
          tay[((t * 4 + k) * 7 + ip) * 7 + j] = (float)v;
        }
  // the density at (s' = 0, zt = 0, zh = 0): the constant term of the surface table
  double rho0 = 0.0;
  for (int i = 0; i < 7; ++i) rho0 += raw[0][0][i][0] * std::pow(s0, i);
  c->e80_s0 = s0;
  c->e80_rho0 = rho0;
  if (cudaMalloc(&c->e80_raw, sizeof(raw)) != cudaSuccess) return NEMO_ERR_NOMEM;
  if (cudaMalloc(&c->e80_tay, tay.size() * sizeof(float)) != cudaSuccess) return NEMO_ERR_NOMEM;
  cudaMemcpy(c->e80_raw, raw, sizeof(raw), cudaMemcpyHostToDevice);
  cudaMemcpy(c->e80_tay, tay.data(), tay.size() * sizeof(float), cudaMemcpyHostToDevice);
  return NEMO_OK;
}

// The sub-step kernel and its grid: one block per 32 x 8 tile, at most all
// co-resident. The mixed form with a linear free surface and the ENE/MIX scheme runs
// k_spg_p2_ene when no block then owns more than P2H_MAXT tiles; otherwise
// k_spg_p2, which keeps its constants in shared memory (ENE/MIX, mixed form) when no
// block owns more than P2_MAXT tiles.
void select_p2(nemo_ctx* c) {
  const long need = (long)((c->jpi + 31) / 32) * ((c->jpj + 7) / 8) * c->nmem;
  const int vvl = !c->nam.ln_linssh;
  const int prec = c->prec;
  auto p2_grid = [&](int cache) {
    const int bps =
        prec == NEMO_PREC_FP64 ? spg_p2_blocks_per_sm<double>(0, vvl) : spg_p2_blocks_per_sm<float>(cache, vvl);
    const long maxb = (long)bps * c->nsm;
    c->p2_blocks = (int)(need < maxb ? need : maxb);
    c->p2_cache = cache;
  };
  const int nv = c->nam.nvor_scheme;
  const bool ene = prec != NEMO_PREC_FP64 && !vvl && (nv == 1 || nv == 5);
  c->p2_hot = 0;
  if (ene && !c->no_p2_hot) {
    const long maxb = (long)spg_p2_ene_blocks_per_sm<float>() * c->nsm;
    if (maxb > 0 && need <= maxb * P2H_MAXT) {
      c->p2_blocks = (int)(need < maxb ? need : maxb);
      c->p2_cache = 1;
      c->p2_hot = 1;
    }
  }
  if (!c->p2_hot) {
    p2_grid(ene ? 1 : 0);
    if (c->p2_cache && (c->p2_blocks < 1 || need > (long)c->p2_blocks * P2_MAXT)) p2_grid(0);
  }
}

int nemo_gpu_create(const nemo_dom_desc* dm, const nemo_namelist* nam, int nmembers, int prec, void* stream,
                    nemo_ctx** out) {
  if (!out) return NEMO_ERR_ARG;
  *out = nullptr;
  if (!dm || !nam) return NEMO_ERR_ARG;
  if (nmembers < 1 || (prec != NEMO_PREC_FP64 && prec != NEMO_PREC_MIXED)) return NEMO_ERR_ARG;
  if (!dm->e1t || !dm->e2t || !dm->e1u || !dm->e2u || !dm->e1v || !dm->e2v || !dm->e1f || !dm->e2f || !dm->ff_f ||
      !dm->ff_t || !dm->k_top || !dm->k_bot || !dm->e3t_0 || !dm->e3u_0 || !dm->e3v_0 || !dm->e3w_0 || !dm->e3f_0)
    return NEMO_ERR_ARG;
  nemo_ctx* c = new nemo_ctx();
  c->jpi = dm->jpi; c->jpj = dm->jpj; c->jpk = dm->jpk; c->nmem = nmembers; c->prec = prec;
  c->n2 = (long)c->jpi * c->jpj; c->n3 = c->n2 * c->jpk;
  c->nam = *nam;
  auto bad = [&](int code) { nemo_gpu_destroy(c); return code; };
  if (dm->jpi < 4 || dm->jpj < 4 || dm->jpk < 3 || dm->jpk > KMAX || dm->jpk > 255) return bad(NEMO_ERR_UNSUPPORTED);
  if (dm->jperio != 0 || nam->ln_isfcav || nam->ln_zad_Aimp) return bad(NEMO_ERR_UNSUPPORTED);
  if (nam->nvor_scheme < 0 || nam->nvor_scheme > 5) return bad(NEMO_ERR_ARG);
  if (nam->ln_traldf_iso && nam->ln_traldf_triad) return bad(NEMO_ERR_ARG);  // one direction of diffusion
  for (int o : {nam->nn_fct_h, nam->nn_fct_v})
    if (o != 0 && o != 2 && o != 4) return bad(NEMO_ERR_ARG);
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return bad(NEMO_ERR_CUDA);
  cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, dev);
  if (stream) c->stream = (cudaStream_t)stream;
  else {
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) return bad(NEMO_ERR_CUDA);
    c->own_stream = true;
  }
  for (auto& st : c->h2d)
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return bad(NEMO_ERR_CUDA);
  for (auto& st : c->d2h)
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return bad(NEMO_ERR_CUDA);
  if (cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking) != cudaSuccess) return bad(NEMO_ERR_CUDA);
  for (cudaEvent_t* e : {&c->ev_main, &c->ev_fork, &c->ev_join})
    if (cudaEventCreateWithFlags(e, cudaEventDisableTiming) != cudaSuccess) return bad(NEMO_ERR_CUDA);
  for (auto& e : c->ev_upf)
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return bad(NEMO_ERR_CUDA);
  for (auto& e : c->ev_h2d)
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return bad(NEMO_ERR_CUDA);
  if (cudaEventCreateWithFlags(&c->ev_spg_done, cudaEventDisableTiming) != cudaSuccess) return bad(NEMO_ERR_CUDA);
  for (auto& e : c->ev_field)
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return bad(NEMO_ERR_CUDA);
  int s = derive_domain(c, dm);
  if (s) { fprintf(stderr, "nemo_gpu_create: %s\n", c->err.c_str()); return bad(s); }
  s = prec == NEMO_PREC_FP64 ? build_dom<double>(c, c->dd) : build_dom<float>(c, c->df);
  if (s) return bad(s);
  const size_t es = prec == NEMO_PREC_FP64 ? 8 : 4;
  const size_t b2 = (size_t)c->n2 * c->nmem * es;
  for (auto& p : c->spg_w) {
    if (cudaMalloc(&p, b2) != cudaSuccess) return bad(NEMO_ERR_NOMEM);
    cudaMemset(p, 0, b2);
  }
  if (!nam->ln_linssh)
    for (auto& p : c->spg_cor) {
      if (cudaMalloc(&p, b2) != cudaSuccess) return bad(NEMO_ERR_NOMEM);
      cudaMemset(p, 0, b2);
    }
  for (auto& p : c->ring) {
    if (cudaMalloc(&p, 4 * b2) != cudaSuccess) return bad(NEMO_ERR_NOMEM);
    cudaMemset(p, 0, 4 * b2);
  }
  for (int w = 0; w < 8; ++w) {
    const size_t bytes = w < 2 ? 2 * b2 : b2;
    if (cudaMalloc(&c->spg_x[w], bytes) != cudaSuccess) return bad(NEMO_ERR_NOMEM);
    cudaMemset(c->spg_x[w], 0, bytes);
  }
  if (prec != NEMO_PREC_FP64) {
    // ten floats a point (k_spg_p2), or three float4 a point (k_spg_p2_ene)
    const size_t bytes = 12 * (size_t)c->nmem * c->n2 * sizeof(float);
    if (cudaMalloc(&c->spg_ff, bytes) != cudaSuccess) return bad(NEMO_ERR_NOMEM);
    cudaMemset(c->spg_ff, 0, bytes);
  }
  if (cudaMalloc(&c->d_wgt1, 3 * (size_t)c->nn_baro * 8) != cudaSuccess) return bad(NEMO_ERR_NOMEM);
  if (cudaMalloc(&c->d_wgt2, 3 * (size_t)c->nn_baro * 8) != cudaSuccess) return bad(NEMO_ERR_NOMEM);
  cudaMemcpy(c->d_wgt1, c->wgt1.data(), c->wgt1.size() * 8, cudaMemcpyHostToDevice);
  cudaMemcpy(c->d_wgt2, c->wgt2.data(), c->wgt2.size() * 8, cudaMemcpyHostToDevice);
  if (cudaMalloc(&c->d_wgtf, 3 * 3 * (size_t)c->nn_baro * 4) != cudaSuccess) return bad(NEMO_ERR_NOMEM);
  float_weights(c);
  cudaMemcpy(c->d_wgtf, c->wgtf.data(), c->wgtf.size() * 4, cudaMemcpyHostToDevice);
  if (cudaMalloc(&c->bar_mem, 2 * sizeof(unsigned int)) != cudaSuccess) return bad(NEMO_ERR_NOMEM);
  if (cudaMalloc(&c->err_flag, sizeof(int)) != cudaSuccess) return bad(NEMO_ERR_NOMEM);
  cudaMemset(c->bar_mem, 0, 2 * sizeof(unsigned int));
  cudaMemset(c->err_flag, 0, sizeof(int));
  select_p2(c);
  if (nam->ln_eos80 && nam->ln_seos) return bad(NEMO_ERR_ARG);  // eos_init: exactly one equation of state
  if (nam->ln_eos80 && upload_eos80(c)) return bad(NEMO_ERR_NOMEM);
  // stp_ctl: one column a thread (at most 2048 blocks of DG_THREADS, then a grid stride)
  c->ctl_nblk = (int)std::min<long>(2048, (c->n2 + DG_THREADS - 1) / DG_THREADS);
  c->hsb_nblk = 2 * c->nsm;
  if (cudaMalloc(&c->ctl_part, (size_t)c->ctl_nblk * c->nmem * CTL_REC * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&c->ctl_out, (size_t)c->nmem * CTL_OUT * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&c->ctl_idx, (size_t)c->nmem * 4 * sizeof(unsigned long long)) != cudaSuccess ||
      cudaMalloc(&c->ctl_flag, sizeof(int)) != cudaSuccess)
    return bad(NEMO_ERR_NOMEM);
  cudaMemset(c->ctl_out, 0, (size_t)c->nmem * CTL_OUT * sizeof(double));
  cudaMemset(c->ctl_flag, 0, sizeof(int));
  for (size_t p = 0; p < (size_t)c->n2; ++p) c->someoce |= c->ssmask[p] == 1.0;
  for (size_t p = 0; p < (size_t)c->n2; ++p)  // a count: exact in any order
    c->usr_zsurf += (1 >= c->ci[p].tlo && 1 <= c->ci[p].thi ? 1.0 : 0.0) * c->tmask_i[p];
  if (c->p2_blocks < 1) return bad(NEMO_ERR_CUDA);
  c->gs_nblk = c->nsm * 4;
  if (cudaMalloc(&c->gs_part, 2 * (size_t)c->gs_nblk * c->nmem * 8) != cudaSuccess) return bad(NEMO_ERR_NOMEM);
  if (cudaMalloc(&c->gs_out, (size_t)c->nmem * 8) != cudaSuccess) return bad(NEMO_ERR_NOMEM);
  // work arrays of the hot path allocated here, so graph capture never allocates
  if (ensure_fct_work(c, 2, c->nam.nn_fct_v == 4)) return bad(NEMO_ERR_NOMEM);
  if ((c->nam.ln_traldf_iso || c->nam.ln_traldf_triad) && ensure_iso_work(c, 2)) return bad(NEMO_ERR_NOMEM);
  if (cudaDeviceSynchronize() != cudaSuccess) return bad(NEMO_ERR_CUDA);
  *out = c;
  return NEMO_OK;
}

int nemo_gpu_destroy(nemo_ctx* c) {
  if (!c) return NEMO_OK;
  if (c->stream) cudaStreamSynchronize(c->stream);
  for (auto& g : c->graphs) cudaGraphExecDestroy(g.second);
  free_dom(c->dd);
  free_dom(c->df);
  for (auto p : c->fct_w) cudaFree(p);
  cudaFree(c->fct_ztw);
  for (auto p : c->iso_w) cudaFree(p);
  for (auto p : c->adj_w) cudaFree(p);
  cudaFree(c->slp_w);
  cudaFree(c->rab_w); cudaFree(c->rab_n); cudaFree(c->zphy_w); cudaFree(c->zdyn_w); cudaFree(c->usr_s); cudaFree(c->fadj_w);
  cudaFree(c->blp_w);
  for (auto p : c->spg_w) cudaFree(p);
  for (auto p : c->spg_cor) cudaFree(p);
  for (auto p : c->ring) cudaFree(p);
  for (auto p : c->spg_x) cudaFree(p);
  cudaFree(c->spg_ff);
  cudaFree(c->d_wgt1); cudaFree(c->d_wgt2); cudaFree(c->d_wgtf);
  cudaFree(c->bar_mem); cudaFree(c->err_flag);
  cudaFree(c->ctl_part); cudaFree(c->ctl_out); cudaFree(c->ctl_idx); cudaFree(c->ctl_flag);
  cudaFree(c->e80_raw); cudaFree(c->e80_tay);
  cudaFree(c->hsb_mem); cudaFree(c->hsb_part); cudaFree(c->hsb_state); cudaFree(c->hsb_out);
  cudaFree(c->gs_part); cudaFree(c->gs_out);
  for (auto e : c->tev)
    if (e) cudaEventDestroy(e);
  for (auto e : c->kc.ev)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : {c->ev_main, c->ev_fork, c->ev_join})
    if (e) cudaEventDestroy(e);
  for (auto e : c->ev_upf)
    if (e) cudaEventDestroy(e);
  for (auto e : c->ev_h2d)
    if (e) cudaEventDestroy(e);
  for (auto p : c->stage) cudaFree(p);
  if (c->ev_spg_done) cudaEventDestroy(c->ev_spg_done);
  if (c->side) cudaStreamDestroy(c->side);
  for (auto e : c->ev_field)
    if (e) cudaEventDestroy(e);
  for (auto st : c->h2d)
    if (st) cudaStreamDestroy(st);
  for (auto st : c->d2h)
    if (st) cudaStreamDestroy(st);
  if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return NEMO_OK;
}

const char* nemo_gpu_last_error(const nemo_ctx* c) { return c ? c->err.c_str() : "null context"; }

int nemo_gpu_synchronize(nemo_ctx* c) {
  if (!c) return NEMO_ERR_ARG;
  for (auto st : c->h2d) CK(cudaStreamSynchronize(st), "synchronize");
  for (auto st : c->d2h) CK(cudaStreamSynchronize(st), "synchronize");
  for (bool& b : c->upf_pending) b = false;
  for (bool& b : c->field_pending) b = false;
  CK(cudaStreamSynchronize(c->stream), "synchronize");
  int flag = 0, blow = 0;
  CK(cudaMemcpy(&blow, c->ctl_flag, sizeof(int), cudaMemcpyDeviceToHost), "read status");
  if (blow) {  // stp_ctl's blow-up test fired (stpctl.F90:149-184)
    cudaMemset(c->ctl_flag, 0, sizeof(int));
    std::vector<double> o((size_t)c->nmem * CTL_OUT);
    CK(cudaMemcpy(o.data(), c->ctl_out, o.size() * sizeof(double), cudaMemcpyDeviceToHost), "read stp_ctl");
    for (int m = 0; m < c->nmem; ++m) {
      const double* z = &o[(size_t)m * CTL_OUT];
      if (z[6] != 0.0)
        return fail(c, NEMO_ERR_BLOWUP,
                    "stp_ctl: |ssh| > 20 m or |U| > 10 m/s or S <= 0 or S >= 100 or NaN (member %d: |ssh| max %g at "
                    "%d %d, |U| max %g at %d %d %d, S min %g at %d %d %d, S max %g at %d %d %d)",
                    m, z[0], (int)z[7], (int)z[8], z[1], (int)z[9], (int)z[10], (int)z[11], -z[2], (int)z[12],
                    (int)z[13], (int)z[14], z[3], (int)z[15], (int)z[16], (int)z[17]);
    }
  }
  CK(cudaMemcpy(&flag, c->err_flag, sizeof(int), cudaMemcpyDeviceToHost), "read status");
  if (flag) {
    cudaMemset(c->err_flag, 0, sizeof(int));
    cudaMemset(c->bar_mem, 0, 2 * sizeof(unsigned int));
    if (flag == TM_ERR) return fail(c, NEMO_ERR_TIMEOUT, "a tensor copy of a TMA-staged tracer kernel did not arrive");
    return fail(c, NEMO_ERR_TIMEOUT, "a grid barrier of the barotropic sub-step kernel timed out");
  }
  return NEMO_OK;
}

int nemo_gpu_bind(nemo_ctx* c, int id, void* p) {
  if (!c || id < 0 || id >= NEMO_F_COUNT) return fail(c, NEMO_ERR_ARG, "bad field id %d", id);
  c->f[id] = p;
  for (auto& g : c->graphs) cudaGraphExecDestroy(g.second);
  c->graphs.clear();
  return NEMO_OK;
}

size_t nemo_gpu_field_numel(const nemo_ctx* c, int id) {
  if (!c || id < 0 || id >= NEMO_F_COUNT) return 0;
  return field_numel(c, id);
}

int nemo_gpu_field_is_fp64(const nemo_ctx* c, int id) {
  if (!c || id == NEMO_F_NMLN) return 0;  // the mixed-layer level is int32
  return c->prec == NEMO_PREC_FP64 || is_fp64_field(id);
}

int nemo_gpu_spg_info(const nemo_ctx* c, int* icycle, int* nn_baro, double* rdtbt) {
  if (!c) return NEMO_ERR_ARG;
  if (icycle) *icycle = c->icycle;
  if (nn_baro) *nn_baro = c->nn_baro;
  if (rdtbt) *rdtbt = c->rdtbt;
  return NEMO_OK;
}

int nemo_gpu_field_upload(nemo_ctx* c, int id, const void* host) {
  if (!c || id < 0 || id >= NEMO_F_COUNT || !host) return fail(c, NEMO_ERR_ARG, "field_upload: bad argument");
  if (!c->f[id]) return fail(c, NEMO_ERR_UNBOUND, "field_upload: field %d is not bound", id);
  size_t bytes = field_numel(c, id) * c->nmem * (nemo_gpu_field_is_fp64(c, id) ? 8 : 4);
  cudaStream_t st = c->h2d[0];
  // A field under 1 MB goes straight into place, after the work already queued and
  // its pending download: for it the device copy out of a staging buffer would cost
  // more than the overlap gains.
  constexpr size_t stage_min_bytes = (size_t)1 << 20;
  if (bytes < stage_min_bytes) {
    CK(cudaEventRecord(c->ev_main, c->stream), "field_upload");
    CK(cudaStreamWaitEvent(st, c->ev_main, 0), "field_upload");
    if (c->field_pending[id]) CK(cudaStreamWaitEvent(st, c->ev_field[id], 0), "field_upload");
    CK(cudaMemcpyAsync(c->f[id], host, bytes, cudaMemcpyHostToDevice, st), "field_upload");
    CK(cudaEventRecord(c->ev_upf[id], st), "field_upload");
    c->upf_pending[id] = true;
    return NEMO_OK;
  }
  if (c->stage_bytes[id] != bytes) {  // the field's staging buffer, made at its first upload
    if (c->stage[id]) {
      CK(cudaStreamSynchronize(c->stream), "field_upload");
      CK(cudaStreamSynchronize(c->side), "field_upload");
      CK(cudaStreamSynchronize(st), "field_upload");
      cudaFree(c->stage[id]);
      c->stage[id] = nullptr;
      c->stage_bytes[id] = 0;
      c->stage_dirty[id] = false;
    }
    if (cudaMalloc(&c->stage[id], bytes) != cudaSuccess)
      return fail(c, NEMO_ERR_NOMEM, "field_upload: staging buffer of %zu bytes", bytes);
    c->stage_bytes[id] = bytes;
  } else if (!c->stage_dirty[id]) {
    // the buffer's previous contents are in the field once its device copy has run
    CK(cudaStreamWaitEvent(st, c->ev_upf[id], 0), "field_upload");
  }
  CK(cudaMemcpyAsync(c->stage[id], host, bytes, cudaMemcpyHostToDevice, st), "field_upload");
  CK(cudaEventRecord(c->ev_h2d[id], st), "field_upload");
  c->stage_dirty[id] = true;
  return NEMO_OK;
}

int nemo_gpu_field_download(nemo_ctx* c, int id, void* host) {
  if (!c || id < 0 || id >= NEMO_F_COUNT || !host) return fail(c, NEMO_ERR_ARG, "field_download: bad argument");
  if (!c->f[id]) return fail(c, NEMO_ERR_UNBOUND, "field_download: field %d is not bound", id);
  size_t bytes = field_numel(c, id) * c->nmem * (nemo_gpu_field_is_fp64(c, id) ? 8 : 4);
  // after the work that writes the field (dyn_spg_ts of the last hot-path step for
  // the fields it writes, else all the work already queued) and the field's upload
  cudaStream_t st = c->d2h[0];
  if (flush_stage(c, c->stream, id)) return NEMO_ERR_CUDA;  // an upload not yet in the field
  if (c->spg_done_valid && spg_writes(id)) {
    CK(cudaStreamWaitEvent(st, c->ev_spg_done, 0), "field_download");
  } else {
    CK(cudaEventRecord(c->ev_main, c->stream), "field_download");
    CK(cudaStreamWaitEvent(st, c->ev_main, 0), "field_download");
  }
  if (c->upf_pending[id]) CK(cudaStreamWaitEvent(st, c->ev_upf[id], 0), "field_download");
  CK(cudaMemcpyAsync(host, c->f[id], bytes, cudaMemcpyDeviceToHost, st), "field_download");
  CK(cudaEventRecord(c->ev_field[id], st), "field_download");
  c->field_pending[id] = true;
  return NEMO_OK;
}

int nemo_gpu_tra_adv_trp(nemo_ctx* c, const void* un, const void* vn, const void* wn, void* zun, void* zvn, void* zwn) {
  if (!c || !un || !vn || !wn || !zun || !zvn || !zwn) return fail(c, NEMO_ERR_ARG, "tra_adv_trp: null pointer");
  if (join_copies(c)) return NEMO_ERR_CUDA;
  cudaError_t e = c->prec == NEMO_PREC_FP64
                      ? launch_adv_trp<double>(dom_now<double>(c), (const double*)un, (const double*)vn,
                                               (const double*)wn, (double*)zun, (double*)zvn, (double*)zwn, c->stream)
                      : launch_adv_trp<float>(dom_now<float>(c), (const float*)un, (const float*)vn, (const float*)wn,
                                              (float*)zun, (float*)zvn, (float*)zwn, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "tra_adv_trp launch");
  return NEMO_OK;
}

// An NVTX range named after the reference routine for the duration of a call, the
// counterpart of timing_start / timing_stop (timing.F90:89-212); free when no tool
// is attached (header-only NVTX v3).
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
};

int nemo_gpu_tra_adv_fct(nemo_ctx* c, int kt, int kit000, const char* cdtype, double p2dt, const void* pun,
                         const void* pvn, const void* pwn, const void* ptb, const void* ptn, void* pta, int kjpt,
                         int kn_fct_h, int kn_fct_v) {
  NvtxRange nvtx_range("tra_adv_fct");
  (void)kt; (void)kit000;
  if (!c) return NEMO_ERR_ARG;
  if (join_copies(c)) return NEMO_ERR_CUDA;
  int is_trc = 0;
  if (int s = check_cdtype(c, cdtype, &is_trc)) return s;
  if (!pun || !pvn || !pwn || !ptb || !ptn || !pta || kjpt < 1) return fail(c, NEMO_ERR_ARG, "tra_adv_fct: bad argument");
  if ((kn_fct_h != 2 && kn_fct_h != 4) || (kn_fct_v != 2 && kn_fct_v != 4))
    return fail(c, NEMO_ERR_ARG, "tra_adv_fct: kn_fct_h/kn_fct_v must be 2 or 4");
  void* tape = c->f[NEMO_F_FCT_TAPE];
  if (tape && c->prec != NEMO_PREC_FP64)
    return fail(c, NEMO_ERR_ARG, "tra_adv_fct: the limiter tape needs an FP64 context");
  return c->prec == NEMO_PREC_FP64
             ? run_fct<double>(c, p2dt, pun, pvn, pwn, 0, ptb, ptn, pta, pta, kjpt, kn_fct_h, kn_fct_v, nullptr, tape)
             : run_fct<float>(c, p2dt, pun, pvn, pwn, 0, ptb, ptn, pta, pta, kjpt, kn_fct_h, kn_fct_v);
}

int nemo_gpu_tra_ldf_lap(nemo_ctx* c, int kt, int kit000, const char* cdtype, const void* pahu, const void* pahv,
                         const void* pgu, const void* pgv, const void* pgui, const void* pgvi, const void* ptb,
                         void* pta, int kjpt, int kpass) {
  NvtxRange nvtx_range("tra_ldf_lap");
  (void)kt; (void)kit000; (void)pgui; (void)pgvi;
  if (!c) return NEMO_ERR_ARG;
  if (join_copies(c)) return NEMO_ERR_CUDA;
  int is_trc = 0;
  if (int s = check_cdtype(c, cdtype, &is_trc)) return s;
  if (!ptb || !pta || kjpt < 1 || (kpass != 1 && kpass != 2)) return fail(c, NEMO_ERR_ARG, "tra_ldf_lap: bad argument");
  if (c->nam.ln_zps && (!pgu || !pgv)) return fail(c, NEMO_ERR_ARG, "tra_ldf_lap: pgu/pgv required with ln_zps");
  return c->prec == NEMO_PREC_FP64 ? run_ldf_lap<double>(c, pahu, pahv, pgu, pgv, ptb, pta, kjpt, kpass)
                                   : run_ldf_lap<float>(c, pahu, pahv, pgu, pgv, ptb, pta, kjpt, kpass);
}

int nemo_gpu_tra_ldf_iso(nemo_ctx* c, int kt, int kit000, const char* cdtype, const void* pahu, const void* pahv,
                         const void* pgu, const void* pgv, const void* pgui, const void* pgvi, const void* ptb,
                         const void* ptbb, void* pta, int kjpt, int kpass) {
  NvtxRange nvtx_range("tra_ldf_iso");
  (void)pgui; (void)pgvi;
  if (!c) return NEMO_ERR_ARG;
  if (join_copies(c)) return NEMO_ERR_CUDA;
  int is_trc = 0;
  if (int s = check_cdtype(c, cdtype, &is_trc)) return s;
  if (!ptb || !ptbb || !pta || kjpt < 1 || (kpass != 1 && kpass != 2))
    return fail(c, NEMO_ERR_ARG, "tra_ldf_iso: bad argument");
  if (c->nam.ln_zps && (!pgu || !pgv)) return fail(c, NEMO_ERR_ARG, "tra_ldf_iso: pgu/pgv required with ln_zps");
  return c->prec == NEMO_PREC_FP64
             ? run_ldf_iso<double>(c, kt, kit000, pahu, pahv, pgu, pgv, ptb, ptbb, pta, kjpt, kpass)
             : run_ldf_iso<float>(c, kt, kit000, pahu, pahv, pgu, pgv, ptb, ptbb, pta, kjpt, kpass);
}

int nemo_gpu_ldf_slp_triad(nemo_ctx* c, int kt, const void* prab_b) {
  (void)kt;
  if (!c) return NEMO_ERR_ARG;
  if (!prab_b) return fail(c, NEMO_ERR_ARG, "ldf_slp_triad: prab_b is NULL");
  if (join_copies(c)) return NEMO_ERR_CUDA;
  for (int id : {NEMO_F_TSB, NEMO_F_GDEPT_N, NEMO_F_GDEPW_N, NEMO_F_NMLN, NEMO_F_TRIADI_G, NEMO_F_TRIADJ_G,
                 NEMO_F_TRIADI, NEMO_F_TRIADJ})
    if (!c->f[id]) return fail(c, NEMO_ERR_UNBOUND, "ldf_slp_triad: field %d must be bound", id);
  cudaError_t e;
  if (c->prec == NEMO_PREC_FP64) {
    TriadArgs<double> a = triad_args<double>(c);
    a.rab = (const double*)prab_b;
    e = launch_ldf_slp_triad<double>(dom_now<double>(c), a, c->stream);
  } else {
    TriadArgs<float> a = triad_args<float>(c);
    a.rab = (const float*)prab_b;
    e = launch_ldf_slp_triad<float>(dom_now<float>(c), a, c->stream);
  }
  if (e != cudaSuccess) return cuda_fail(c, e, "ldf_slp_triad launch");
  return NEMO_OK;
}


int nemo_gpu_tra_ldf_triad(nemo_ctx* c, int kt, int kit000, const char* cdtype, const void* pahu, const void* pahv,
                           const void* pgu, const void* pgv, const void* pgui, const void* pgvi, const void* ptb,
                           const void* ptbb, void* pta, int kjpt, int kpass) {
  NvtxRange nvtx_range("tra_ldf_triad");
  (void)pgu; (void)pgv; (void)pgui; (void)pgvi;
  if (!c) return NEMO_ERR_ARG;
  if (join_copies(c)) return NEMO_ERR_CUDA;
  int is_trc = 0;
  if (int s = check_cdtype(c, cdtype, &is_trc)) return s;
  if (!ptb || !pta || kjpt < 1 || (kpass != 1 && kpass != 2) || (kpass == 2 && !ptbb))
    return fail(c, NEMO_ERR_ARG, "tra_ldf_triad: bad argument");
  for (int id : {NEMO_F_AH_WSLP2, NEMO_F_AKZ, NEMO_F_TRIADI_G, NEMO_F_TRIADJ_G, NEMO_F_TRIADI, NEMO_F_TRIADJ,
                 NEMO_F_GDEPT_N})
    if (!c->f[id]) return fail(c, NEMO_ERR_UNBOUND, "tra_ldf_triad: field %d must be bound", id);
  return c->prec == NEMO_PREC_FP64 ? run_ldf_triad<double>(c, kt, kit000, pahu, pahv, ptb, ptbb, pta, kjpt, kpass)
                                   : run_ldf_triad<float>(c, kt, kit000, pahu, pahv, ptb, ptbb, pta, kjpt, kpass);
}

int nemo_gpu_tra_ldf_blp(nemo_ctx* c, int kt, int kit000, const char* cdtype, const void* pahu, const void* pahv,
                         const void* pgu, const void* pgv, const void* pgui, const void* pgvi, const void* ptb,
                         void* pta, int kjpt, int kldf) {
  NvtxRange nvtx_range("tra_ldf_blp");
  (void)pgui; (void)pgvi;
  if (!c) return NEMO_ERR_ARG;
  if (join_copies(c)) return NEMO_ERR_CUDA;
  int is_trc = 0;
  if (int s = check_cdtype(c, cdtype, &is_trc)) return s;
  if (!ptb || !pta || kjpt < 1) return fail(c, NEMO_ERR_ARG, "tra_ldf_blp: bad argument");
  if (kldf != 20 && kldf != 21 && kldf != 22)
    return fail(c, NEMO_ERR_UNSUPPORTED, "tra_ldf_blp: kldf 20 (iso-level), 21 (rotated) or 22 (triad) only");
  if (kldf == 22)
    for (int id : {NEMO_F_AH_WSLP2, NEMO_F_AKZ, NEMO_F_TRIADI_G, NEMO_F_TRIADJ_G, NEMO_F_TRIADI, NEMO_F_TRIADJ,
                   NEMO_F_GDEPT_N})
      if (!c->f[id]) return fail(c, NEMO_ERR_UNBOUND, "tra_ldf_blp: field %d must be bound (triad)", id);
  if (c->nam.ln_zps && (!pgu || !pgv)) return fail(c, NEMO_ERR_ARG, "tra_ldf_blp: pgu/pgv required with ln_zps");
  return c->prec == NEMO_PREC_FP64 ? run_ldf_blp<double>(c, kt, kit000, pahu, pahv, pgu, pgv, ptb, pta, kjpt, kldf)
                                   : run_ldf_blp<float>(c, kt, kit000, pahu, pahv, pgu, pgv, ptb, pta, kjpt, kldf);
}

int nemo_gpu_zps_hde(nemo_ctx* c, int kt, int kjpt, const void* pta, void* pgtu, void* pgtv) {
  (void)kt;
  if (!c) return NEMO_ERR_ARG;
  if (!pta || !pgtu || !pgtv || kjpt < 1) return fail(c, NEMO_ERR_ARG, "zps_hde: bad argument");
  if (join_copies(c)) return NEMO_ERR_CUDA;
  cudaError_t e = c->prec == NEMO_PREC_FP64
                      ? launch_zps_hde<double>(dom_now<double>(c), (const double*)pta, (double*)pgtu, (double*)pgtv,
                                               kjpt, c->stream)
                      : launch_zps_hde<float>(dom_now<float>(c), (const float*)pta, (float*)pgtu, (float*)pgtv, kjpt,
                                              c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "zps_hde launch");
  return NEMO_OK;
}

int nemo_gpu_zps_hde_rd(nemo_ctx* c, int kt, const void* pts, const void* prd, void* pgru, void* pgrv) {
  (void)kt;
  if (!c) return NEMO_ERR_ARG;
  if (!pts || !prd || !pgru || !pgrv) return fail(c, NEMO_ERR_ARG, "zps_hde_rd: null array");
  if (join_copies(c)) return NEMO_ERR_CUDA;
  if (!c->nam.ln_seos && !c->nam.ln_eos80)
    return fail(c, NEMO_ERR_UNSUPPORTED, "zps_hde_rd: needs an equation of state (ln_seos or ln_eos80)");
  if (!c->f[NEMO_F_GDEPT_N]) return fail(c, NEMO_ERR_UNBOUND, "zps_hde_rd: gdept_n must be bound");
  cudaError_t e;
  if (c->prec == NEMO_PREC_FP64) {
    EosArgs<double> a = eos_args<double>(c, 0);
    a.pts = (const double*)pts;
    e = launch_zps_hde_rd<double>(dom_now<double>(c), a, (const double*)prd, (double*)pgru, (double*)pgrv, c->stream);
  } else {
    EosArgs<float> a = eos_args<float>(c, 0);
    a.pts = (const float*)pts;
    e = launch_zps_hde_rd<float>(dom_now<float>(c), a, (const float*)prd, (float*)pgru, (float*)pgrv, c->stream);
  }
  if (e != cudaSuccess) return cuda_fail(c, e, "zps_hde_rd launch");
  return NEMO_OK;
}

int nemo_gpu_tra_zdf_imp(nemo_ctx* c, int kt, int kit000, const char* cdtype, double p2dt, const void* ptb, void* pta,
                         int kjpt) {
  NvtxRange nvtx_range("tra_zdf_imp");
  (void)kt; (void)kit000;
  if (!c) return NEMO_ERR_ARG;
  if (join_copies(c)) return NEMO_ERR_CUDA;
  int is_trc = 0;
  if (int s = check_cdtype(c, cdtype, &is_trc)) return s;
  if (!ptb || !pta || kjpt < 1) return fail(c, NEMO_ERR_ARG, "tra_zdf_imp: bad argument");
  return c->prec == NEMO_PREC_FP64 ? run_zdf<double>(c, p2dt, ptb, pta, kjpt, is_trc, 0)
                                   : run_zdf<float>(c, p2dt, ptb, pta, kjpt, is_trc, 0);
}

int nemo_gpu_tra_zdf(nemo_ctx* c, int kt) {
  if (!c) return NEMO_ERR_ARG;
  if (join_copies(c)) return NEMO_ERR_CUDA;
  const nemo_namelist& nm = c->nam;
  if (!c->f[NEMO_F_TSB] || !c->f[NEMO_F_TSA]) return fail(c, NEMO_ERR_UNBOUND, "tra_zdf: tsb and tsa must be bound");
  if (nm.neuler == 0 && kt == nm.nit000) c->r2dt = nm.rn_rdt;
  else if (kt <= nm.nit000 + 1 || c->r2dt == 0.0) c->r2dt = 2.0 * nm.rn_rdt;
  int s = c->prec == NEMO_PREC_FP64 ? run_zdf<double>(c, c->r2dt, c->f[NEMO_F_TSB], c->f[NEMO_F_TSA], 2, 0, 0)
                                    : run_zdf<float>(c, c->r2dt, c->f[NEMO_F_TSB], c->f[NEMO_F_TSA], 2, 0, 0);
  if (s) return s;
  // WHERE( tsa(:,:,:,jp_sal) < 0 ) tsa = 0.1 on every member's salinity slice
  for (int m = 0; m < c->nmem; ++m) {
    cudaError_t e = c->prec == NEMO_PREC_FP64
                        ? launch_clamp<double>((double*)c->f[NEMO_F_TSA] + (2L * m + 1) * c->n3, c->n3, c->stream)
                        : launch_clamp<float>((float*)c->f[NEMO_F_TSA] + (2L * m + 1) * c->n3, c->n3, c->stream);
    if (e != cudaSuccess) return cuda_fail(c, e, "tra_zdf clamp");
  }
  return NEMO_OK;
}

int nemo_gpu_tra_nxt(nemo_ctx* c, int kt) {
  if (!c) return NEMO_ERR_ARG;
  if (join_copies(c)) return NEMO_ERR_CUDA;
  const nemo_namelist& nm = c->nam;
  void* const* F = c->f;
  if (!F[NEMO_F_TSB] || !F[NEMO_F_TSN] || !F[NEMO_F_TSA])
    return fail(c, NEMO_ERR_UNBOUND, "tra_nxt: tsb, tsn and tsa must be bound");
  if (!nm.ln_linssh) {  // tra_nxt_vvl
    if (int s = vvl_check(c, "tra_nxt", {NEMO_F_E3T_B, NEMO_F_E3T_N, NEMO_F_E3T_A, NEMO_F_EMP, NEMO_F_EMP_B,
                                         NEMO_F_SBC_TSC, NEMO_F_SBC_TSC_B}))
      return s;
    if (nm.ln_traqsr && (!F[NEMO_F_QSR_HC] || !F[NEMO_F_QSR_HC_B]))
      return fail(c, NEMO_ERR_UNBOUND, "tra_nxt: qsr_hc and qsr_hc_b must be bound with ln_traqsr");
    return c->prec == NEMO_PREC_FP64 ? run_vvl<double>(c, kt, VVL_TRA_NXT) : run_vvl<float>(c, kt, VVL_TRA_NXT);
  }
  return c->prec == NEMO_PREC_FP64 ? run_tra_nxt<double>(c, kt) : run_tra_nxt<float>(c, kt);
}

int nemo_gpu_ldf_slp(nemo_ctx* c, int kt, const void* prd, const void* pn2) {
  NvtxRange nvtx_range("ldf_slp");
  (void)kt;
  if (!c) return NEMO_ERR_ARG;
  if (!prd || !pn2) return fail(c, NEMO_ERR_ARG, "ldf_slp: null prd or pn2");
  if (join_copies(c)) return NEMO_ERR_CUDA;
  for (int id : {NEMO_F_USLP, NEMO_F_VSLP, NEMO_F_WSLPI, NEMO_F_WSLPJ, NEMO_F_GDEPT_N, NEMO_F_GDEPW_N, NEMO_F_NMLN,
                 NEMO_F_HMLP, NEMO_F_HMLPT})
    if (!c->f[id]) return fail(c, NEMO_ERR_UNBOUND, "ldf_slp: field %d must be bound", id);
  const nemo_namelist& nm = c->nam;
  if (nm.ln_isfcav || nm.ln_sco)
    return fail(c, NEMO_ERR_UNSUPPORTED, "ldf_slp: z-coordinate without cavities only");
  return c->prec == NEMO_PREC_FP64 ? run_ldf_slp<double>(c, prd, pn2) : run_ldf_slp<float>(c, prd, pn2);
}

int nemo_gpu_zdf_mxl(nemo_ctx* c, int kt) {
  (void)kt;
  if (!c) return NEMO_ERR_ARG;
  if (join_copies(c)) return NEMO_ERR_CUDA;
  for (int id : {NEMO_F_RN2B, NEMO_F_AVT, NEMO_F_GDEPT_N, NEMO_F_GDEPW_N, NEMO_F_NMLN, NEMO_F_HMLP, NEMO_F_HMLPT})
    if (!c->f[id]) return fail(c, NEMO_ERR_UNBOUND, "zdf_mxl: field %d must be bound", id);
  return c->prec == NEMO_PREC_FP64 ? run_zdf_mxl<double>(c) : run_zdf_mxl<float>(c);
}

int nemo_gpu_usrdef_sbc(nemo_ctx* c, int kt) {
  if (!c) return NEMO_ERR_ARG;
  if (join_copies(c)) return NEMO_ERR_CUDA;
  if (int s = usr_check(c)) return s;
  if (int s = usr_put(c, kt)) return s;
  return c->prec == NEMO_PREC_FP64 ? run_usrdef_sbc<double>(c) : run_usrdef_sbc<float>(c);
}

int nemo_gpu_zdf_phy(nemo_ctx* c, int kt) {
  (void)kt;
  if (!c) return NEMO_ERR_ARG;
  if (join_copies(c)) return NEMO_ERR_CUDA;
  if (int s = zphy_check(c)) return s;
  return c->prec == NEMO_PREC_FP64 ? run_zdf_phy<double>(c) : run_zdf_phy<float>(c);
}

int nemo_gpu_dyn_keg(nemo_ctx* c, int kt, int kscheme) {
  (void)kt;
  if (!c) return NEMO_ERR_ARG;
  if (join_copies(c)) return NEMO_ERR_CUDA;
  for (int id : {NEMO_F_UN, NEMO_F_VN, NEMO_F_UA, NEMO_F_VA})
    if (!c->f[id]) return fail(c, NEMO_ERR_UNBOUND, "dyn_keg: un, vn, ua and va must be bound");
  if (kscheme != 0) return fail(c, NEMO_ERR_UNSUPPORTED, "dyn_keg: the centred scheme (nkeg_C2) only");
  void* const* F = c->f;
  cudaError_t e = c->prec == NEMO_PREC_FP64
                      ? launch_dyn_keg<double>(dom_now<double>(c), (const double*)F[NEMO_F_UN], (const double*)F[NEMO_F_VN],
                                               (double*)F[NEMO_F_UA], (double*)F[NEMO_F_VA], c->stream)
                      : launch_dyn_keg<float>(dom_now<float>(c), (const float*)F[NEMO_F_UN], (const float*)F[NEMO_F_VN],
                                              (float*)F[NEMO_F_UA], (float*)F[NEMO_F_VA], c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "dyn_keg launch");
  return NEMO_OK;
}

int nemo_gpu_dyn_zad(nemo_ctx* c, int kt) {
  (void)kt;
  if (!c) return NEMO_ERR_ARG;
  if (join_copies(c)) return NEMO_ERR_CUDA;
  for (int id : {NEMO_F_UN, NEMO_F_VN, NEMO_F_WN, NEMO_F_UA, NEMO_F_VA})
    if (!c->f[id]) return fail(c, NEMO_ERR_UNBOUND, "dyn_zad: un, vn, wn, ua and va must be bound");
  void* const* F = c->f;
  cudaError_t e = c->prec == NEMO_PREC_FP64
                      ? launch_dyn_zad<double>(dom_now<double>(c), (const double*)F[NEMO_F_UN], (const double*)F[NEMO_F_VN],
                                               (const double*)F[NEMO_F_WN], (double*)F[NEMO_F_UA],
                                               (double*)F[NEMO_F_VA], c->stream)
                      : launch_dyn_zad<float>(dom_now<float>(c), (const float*)F[NEMO_F_UN], (const float*)F[NEMO_F_VN],
                                              (const float*)F[NEMO_F_WN], (float*)F[NEMO_F_UA], (float*)F[NEMO_F_VA],
                                              c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "dyn_zad launch");
  return NEMO_OK;
}

int nemo_gpu_vor_ene(nemo_ctx* c, int kt, int kvor, const void* pun, const void* pvn, void* pua, void* pva) {
  (void)kt;
  if (!c) return NEMO_ERR_ARG;
  if (join_copies(c)) return NEMO_ERR_CUDA;
  if (!pun || !pvn || !pua || !pva) return fail(c, NEMO_ERR_ARG, "vor_ene: null array");
  if (kvor != 1 && kvor != 2 && kvor != 4)
    return fail(c, NEMO_ERR_UNSUPPORTED, "vor_ene: kvor %d (the flux-form metric terms are not included)", kvor);
  if (c->nam.ln_sco) return fail(c, NEMO_ERR_UNSUPPORTED, "vor_ene: z-coordinate only");
  cudaError_t e = c->prec == NEMO_PREC_FP64
                      ? launch_vor_ene<double>(dom_now<double>(c), kvor, (const double*)pun, (const double*)pvn,
                                               (double*)pua, (double*)pva, c->stream)
                      : launch_vor_ene<float>(dom_now<float>(c), kvor, (const float*)pun, (const float*)pvn,
                                              (float*)pua, (float*)pva, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "vor_ene launch");
  return NEMO_OK;
}

int nemo_gpu_dyn_ldf_lap(nemo_ctx* c, int kt, const void* pub, const void* pvb, void* pua, void* pva, int kpass) {
  (void)kt;
  if (!c) return NEMO_ERR_ARG;
  if (join_copies(c)) return NEMO_ERR_CUDA;
  if (!pub || !pvb || !pua || !pva || (kpass != 1 && kpass != 2)) return fail(c, NEMO_ERR_ARG, "dyn_ldf_lap: bad argument");
  if (!c->f[NEMO_F_AHMT] || !c->f[NEMO_F_AHMF]) return fail(c, NEMO_ERR_UNBOUND, "dyn_ldf_lap: ahmt and ahmf must be bound");
  if (!c->nam.ln_linssh) return fail(c, NEMO_ERR_UNSUPPORTED, "dyn_ldf_lap: linear free surface only");
  cudaError_t e;
  if (c->prec == NEMO_PREC_FP64)
    e = launch_dyn_ldf_lap<double>(dom_now<double>(c), (const double*)c->f[NEMO_F_AHMT], (const double*)c->f[NEMO_F_AHMF],
                                   (const double*)pub, (const double*)pvb, (double*)pua, (double*)pva,
                                   kpass == 1 ? 1.0 : -1.0, c->stream);
  else
    e = launch_dyn_ldf_lap<float>(dom_now<float>(c), (const float*)c->f[NEMO_F_AHMT], (const float*)c->f[NEMO_F_AHMF],
                                  (const float*)pub, (const float*)pvb, (float*)pua, (float*)pva,
                                  kpass == 1 ? 1.f : -1.f, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "dyn_ldf_lap launch");
  return NEMO_OK;
}

static int eos_check(nemo_ctx* c, const char* what) {
  if (!c) return NEMO_ERR_ARG;
  if (!c->nam.ln_seos && !c->nam.ln_eos80)
    return fail(c, NEMO_ERR_UNSUPPORTED, "%s: the simplified (ln_seos) or EOS-80 (ln_eos80) equation of state", what);
  if (join_copies(c)) return NEMO_ERR_CUDA;
  return NEMO_OK;
}

int nemo_gpu_eos_insitu(nemo_ctx* c, const void* pts, void* prd, const void* pdep) {
  if (int s = eos_check(c, "eos_insitu")) return s;
  if (!pts || !prd || !pdep) return fail(c, NEMO_ERR_ARG, "eos_insitu: null array");
  return c->prec == NEMO_PREC_FP64 ? run_eos<double>(c, 0, pts, prd, nullptr, pdep, nullptr, nullptr, nullptr)
                                   : run_eos<float>(c, 0, pts, prd, nullptr, pdep, nullptr, nullptr, nullptr);
}

int nemo_gpu_eos_insitu_pot(nemo_ctx* c, const void* pts, void* prd, void* prhop, const void* pdep) {
  if (int s = eos_check(c, "eos_insitu_pot")) return s;
  if (!pts || !prd || !prhop || !pdep) return fail(c, NEMO_ERR_ARG, "eos_insitu_pot: null array");
  return c->prec == NEMO_PREC_FP64 ? run_eos<double>(c, 1, pts, prd, prhop, pdep, nullptr, nullptr, nullptr)
                                   : run_eos<float>(c, 1, pts, prd, prhop, pdep, nullptr, nullptr, nullptr);
}

int nemo_gpu_rab_3d(nemo_ctx* c, const void* pts, void* pab) {
  if (int s = eos_check(c, "rab_3d")) return s;
  if (!pts || !pab) return fail(c, NEMO_ERR_ARG, "rab_3d: null array");
  if (!c->f[NEMO_F_GDEPT_N]) return fail(c, NEMO_ERR_UNBOUND, "rab_3d: gdept_n must be bound");
  return c->prec == NEMO_PREC_FP64 ? run_eos<double>(c, 2, pts, nullptr, nullptr, nullptr, pab, nullptr, nullptr)
                                   : run_eos<float>(c, 2, pts, nullptr, nullptr, nullptr, pab, nullptr, nullptr);
}

int nemo_gpu_bn2(nemo_ctx* c, const void* pts, const void* pab, void* pn2) {
  if (!c) return NEMO_ERR_ARG;
  if (join_copies(c)) return NEMO_ERR_CUDA;
  if (!pts || !pab || !pn2) return fail(c, NEMO_ERR_ARG, "bn2: null array");
  if (!c->f[NEMO_F_GDEPT_N] || !c->f[NEMO_F_GDEPW_N])
    return fail(c, NEMO_ERR_UNBOUND, "bn2: gdept_n and gdepw_n must be bound");
  return c->prec == NEMO_PREC_FP64 ? run_eos<double>(c, 3, pts, nullptr, nullptr, nullptr, nullptr, pab, pn2)
                                   : run_eos<float>(c, 3, pts, nullptr, nullptr, nullptr, nullptr, pab, pn2);
}

int nemo_gpu_dyn_hpg(nemo_ctx* c, int kt) {
  (void)kt;
  if (!c) return NEMO_ERR_ARG;
  if (join_copies(c)) return NEMO_ERR_CUDA;
  if (!c->f[NEMO_F_RHD] || !c->f[NEMO_F_UA] || !c->f[NEMO_F_VA])
    return fail(c, NEMO_ERR_UNBOUND, "dyn_hpg: rhd, ua and va must be bound");
  if (c->nam.ln_zps || c->nam.ln_sco || c->nam.ln_isfcav)
    return fail(c, NEMO_ERR_UNSUPPORTED, "dyn_hpg: z-coordinate with full steps only (hpg_zco)");
  return c->prec == NEMO_PREC_FP64 ? run_dyn_hpg<double>(c) : run_dyn_hpg<float>(c);
}

int nemo_gpu_tra_sbc(nemo_ctx* c, int kt) {
  if (!c) return NEMO_ERR_ARG;
  if (join_copies(c)) return NEMO_ERR_CUDA;
  if (!sbc_bound(c) || !c->f[NEMO_F_TSN] || !c->f[NEMO_F_TSA])
    return fail(c, NEMO_ERR_UNBOUND, "tra_sbc: qns, qsr, emp, sfx, sbc_tsc, sbc_tsc_b, tsn and tsa must be bound");
  return c->prec == NEMO_PREC_FP64 ? run_tra_sbc<double>(c, kt) : run_tra_sbc<float>(c, kt);
}

int nemo_gpu_tra_qsr(nemo_ctx* c, int kt) {
  if (!c) return NEMO_ERR_ARG;
  if (join_copies(c)) return NEMO_ERR_CUDA;
  if (!c->nam.ln_traqsr) return fail(c, NEMO_ERR_ARG, "tra_qsr: ln_traqsr is off");
  if (!qsr_bound(c) || !c->f[NEMO_F_TSA])
    return fail(c, NEMO_ERR_UNBOUND, "tra_qsr: qsr, gdepw_n, qsr_hc, qsr_hc_b, fraqsr_1lev and tsa must be bound");
  return c->prec == NEMO_PREC_FP64 ? run_tra_qsr<double>(c, kt) : run_tra_qsr<float>(c, kt);
}

int nemo_gpu_wzv(nemo_ctx* c, int kt) {
  if (!c) return NEMO_ERR_ARG;
  if (join_copies(c)) return NEMO_ERR_CUDA;
  if (!c->f[NEMO_F_UN] || !c->f[NEMO_F_VN] || !c->f[NEMO_F_WN])
    return fail(c, NEMO_ERR_UNBOUND, "wzv: un, vn and wn must be bound");
  return c->prec == NEMO_PREC_FP64 ? run_wzv<double>(c, kt) : run_wzv<float>(c, kt);
}

int nemo_gpu_dyn_zdf_step(nemo_ctx* c, int kt) {
  if (!c) return NEMO_ERR_ARG;
  if (join_copies(c)) return NEMO_ERR_CUDA;
  if (int s = dyn_zdf_check(c)) return s;
  return c->prec == NEMO_PREC_FP64 ? run_dyn_zdf_step<double>(c, kt) : run_dyn_zdf_step<float>(c, kt);
}

int nemo_gpu_dyn_nxt(nemo_ctx* c, int kt) {
  if (!c) return NEMO_ERR_ARG;
  if (join_copies(c)) return NEMO_ERR_CUDA;
  if (!c->nam.ln_linssh) {
    if (!c->nam.ln_bt_fw) return fail(c, NEMO_ERR_UNSUPPORTED, "dyn_nxt: ln_bt_fw only");
    if (int s = vvl_check(c, "dyn_nxt",
                          {NEMO_F_UN, NEMO_F_VN, NEMO_F_UA, NEMO_F_VA, NEMO_F_UB, NEMO_F_VB, NEMO_F_UN_B, NEMO_F_VN_B,
                           NEMO_F_UB_B, NEMO_F_VB_B, NEMO_F_UA_B, NEMO_F_VA_B, NEMO_F_E3T_B, NEMO_F_E3T_N,
                           NEMO_F_E3T_A, NEMO_F_E3U_N, NEMO_F_E3V_N, NEMO_F_E3U_A, NEMO_F_E3V_A, NEMO_F_E3U_B,
                           NEMO_F_E3V_B, NEMO_F_R1_HU_A, NEMO_F_R1_HV_A, NEMO_F_R1_HU_N, NEMO_F_R1_HV_N, NEMO_F_HU_B,
                           NEMO_F_HV_B, NEMO_F_R1_HU_B, NEMO_F_R1_HV_B, NEMO_F_EMP, NEMO_F_EMP_B}))
      return s;
    return c->prec == NEMO_PREC_FP64 ? run_vvl<double>(c, kt, VVL_DYN_NXT) : run_vvl<float>(c, kt, VVL_DYN_NXT);
  }
  if (int s = model_fields(c, "dyn_nxt")) return s;
  return c->prec == NEMO_PREC_FP64 ? run_dyn_nxt<double>(c, kt) : run_dyn_nxt<float>(c, kt);
}

// ---------------------------------------------------------------- stp_ctl, dia_hsb
int nemo_gpu_stp_ctl(nemo_ctx* c, int kt) {
  (void)kt;
  if (!c) return NEMO_ERR_ARG;
  if (join_copies(c)) return NEMO_ERR_CUDA;
  if (!c->f[NEMO_F_SSHN] || !c->f[NEMO_F_UN] || !c->f[NEMO_F_TSN])
    return fail(c, NEMO_ERR_UNBOUND, "stp_ctl: sshn, un and tsn must be bound");
  return c->prec == NEMO_PREC_FP64 ? run_stp_ctl<double>(c) : run_stp_ctl<float>(c);
}

int nemo_gpu_stp_ctl_result(nemo_ctx* c, double* zmax, int* loc, int* kindic) {
  if (!c) return NEMO_ERR_ARG;
  CK(cudaStreamSynchronize(c->stream), "stp_ctl result");
  std::vector<double> o((size_t)c->nmem * CTL_OUT);
  CK(cudaMemcpy(o.data(), c->ctl_out, o.size() * sizeof(double), cudaMemcpyDeviceToHost), "stp_ctl result");
  for (int m = 0; m < c->nmem; ++m) {
    const double* z = &o[(size_t)m * CTL_OUT];
    if (zmax)
      for (int t = 0; t < NEMO_CTL_N; ++t) zmax[(size_t)m * NEMO_CTL_N + t] = z[t];
    if (kindic) kindic[m] = (int)z[6];
    if (loc)
      for (int t = 0; t < NEMO_CTL_NLOC; ++t) loc[(size_t)m * NEMO_CTL_NLOC + t] = (int)z[7 + t];
  }
  return NEMO_OK;
}

int nemo_gpu_dia_hsb_init(nemo_ctx* c) {
  if (!c) return NEMO_ERR_ARG;
  if (join_copies(c)) return NEMO_ERR_CUDA;
  if (!c->f[NEMO_F_SSHN] || !c->f[NEMO_F_TSN])
    return fail(c, NEMO_ERR_UNBOUND, "dia_hsb_init: sshn and tsn must be bound");
  const size_t n2 = c->n2, n3 = c->n3, nm = c->nmem;
  if (!c->hsb_mem) {
    const size_t words = 2 * n2 + 3 * nm * n2 + 3 * nm * n3;
    if (cudaMalloc(&c->hsb_mem, words * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&c->hsb_part, (size_t)c->hsb_nblk * nm * HSB_NS * 2 * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&c->hsb_state, nm * 8 * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&c->hsb_out, nm * NEMO_HSB_N * sizeof(double)) != cudaSuccess)
      return fail(c, NEMO_ERR_NOMEM, "dia_hsb work arrays");
    CK(cudaMemset(c->hsb_mem, 0, words * sizeof(double)), "dia_hsb = 0");
  }
  // surf = e1e2t * tmask_i (diahsb.F90:411), tmask_h (dommsk.F90:213-217, closed
  // domain), surf_tot = glob_sum(surf) with DDPDD (:412)
  std::vector<double> h(2 * n2);
  double re = 0.0, im = 0.0;
  for (size_t p = 0; p < n2; ++p) {
    h[p] = c->e1e2t[p] * c->tmask_i[p];
    const int ji = (int)(p % c->jpi) + 1, jj = (int)(p / c->jpi) + 1;
    h[n2 + p] = (ji == 1 || ji == c->jpi || jj == 1 || jj == c->jpj) ? 0.0 : 1.0;
    const double a = h[p] * c->tmask_i[p];  // DDPDD (lib_fortran.F90:300-332)
    const double zt1 = a + re, zerr = zt1 - a;
    const double zt2 = ((re - zerr) + (a - (zt1 - zerr))) + 0.0 + im;
    const double sum = zt1 + zt2;
    im = zt2 - ((zt1 + zt2) - zt1);
    re = sum;
  }
  CK(cudaMemcpy(c->hsb_mem, h.data(), 2 * n2 * sizeof(double), cudaMemcpyHostToDevice), "dia_hsb surf");
  std::vector<double> st(nm * 8, 0.0);
  for (size_t m = 0; m < nm; ++m) st[m * 8 + 5] = re;
  CK(cudaMemcpy(c->hsb_state, st.data(), st.size() * sizeof(double), cudaMemcpyHostToDevice), "dia_hsb state");
  CK(cudaMemset(c->hsb_out, 0, nm * NEMO_HSB_N * sizeof(double)), "dia_hsb out");
  cudaError_t e = c->prec == NEMO_PREC_FP64
                      ? launch_hsb_init<double>(dom<double>(c), hsb_args<double>(c), 4 * c->nsm, c->stream)
                      : launch_hsb_init<float>(dom<float>(c), hsb_args<float>(c), 4 * c->nsm, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "dia_hsb_init launch");
  c->hsb_on = true;
  for (auto& g : c->graphs) cudaGraphExecDestroy(g.second);  // the model step now runs dia_hsb
  c->graphs.clear();
  return NEMO_OK;
}

int nemo_gpu_dia_hsb(nemo_ctx* c, int kt) {
  (void)kt;
  if (!c) return NEMO_ERR_ARG;
  if (join_copies(c)) return NEMO_ERR_CUDA;
  int s = hsb_check(c);
  if (s) return s;
  return c->prec == NEMO_PREC_FP64 ? run_dia_hsb<double>(c) : run_dia_hsb<float>(c);
}

int nemo_gpu_dia_hsb_result(nemo_ctx* c, double* out) {
  if (!c || !out) return NEMO_ERR_ARG;
  if (!c->hsb_on) return fail(c, NEMO_ERR_STATE, "dia_hsb_result: no dia_hsb yet");
  CK(cudaStreamSynchronize(c->stream), "dia_hsb result");
  CK(cudaMemcpy(out, c->hsb_out, (size_t)c->nmem * NEMO_HSB_N * sizeof(double), cudaMemcpyDeviceToHost),
     "dia_hsb result");
  return NEMO_OK;
}

int nemo_gpu_ssh_swp(nemo_ctx* c, int kt) {
  if (!c) return NEMO_ERR_ARG;
  if (join_copies(c)) return NEMO_ERR_CUDA;
  if (!c->f[NEMO_F_SSHB] || !c->f[NEMO_F_SSHN] || !c->f[NEMO_F_SSHA])
    return fail(c, NEMO_ERR_UNBOUND, "ssh_swp: sshb, sshn and ssha must be bound");
  if (!c->nam.ln_linssh) {
    if (int s = vvl_check(c, "ssh_swp", {NEMO_F_EMP, NEMO_F_EMP_B})) return s;
    return c->prec == NEMO_PREC_FP64 ? run_vvl<double>(c, kt, VVL_SSH_SWP) : run_vvl<float>(c, kt, VVL_SSH_SWP);
  }
  return c->prec == NEMO_PREC_FP64 ? run_ssh_swp<double>(c, kt) : run_ssh_swp<float>(c, kt);
}

int nemo_gpu_dom_vvl_sf_nxt(nemo_ctx* c, int kt) {
  if (!c) return NEMO_ERR_ARG;
  if (join_copies(c)) return NEMO_ERR_CUDA;
  if (int s = vvl_check(c, "dom_vvl_sf_nxt",
                        {NEMO_F_SSHA, NEMO_F_SSHB, NEMO_F_SSHN, NEMO_F_E3T_B, NEMO_F_E3T_N, NEMO_F_E3T_A, NEMO_F_E3U_A,
                         NEMO_F_E3V_A, NEMO_F_HU_A, NEMO_F_HV_A, NEMO_F_R1_HU_A, NEMO_F_R1_HV_A}))
    return s;
  return c->prec == NEMO_PREC_FP64 ? run_vvl<double>(c, kt, VVL_SF_NXT) : run_vvl<float>(c, kt, VVL_SF_NXT);
}

int nemo_gpu_dom_vvl_sf_swp(nemo_ctx* c, int kt) {
  if (!c) return NEMO_ERR_ARG;
  if (join_copies(c)) return NEMO_ERR_CUDA;
  if (int s = vvl_check(c, "dom_vvl_sf_swp",
                        {NEMO_F_E3T_B, NEMO_F_E3T_N, NEMO_F_E3T_A, NEMO_F_E3U_N, NEMO_F_E3V_N, NEMO_F_E3W_N,
                         NEMO_F_E3U_A, NEMO_F_E3V_A, NEMO_F_SSHN, NEMO_F_HU_A, NEMO_F_HV_A, NEMO_F_R1_HU_A,
                         NEMO_F_R1_HV_A, NEMO_F_HU_N, NEMO_F_HV_N, NEMO_F_R1_HU_N, NEMO_F_R1_HV_N, NEMO_F_HT_N}))
    return s;
  void* const* F = c->f;
  if ((F[NEMO_F_E3UW_N] || F[NEMO_F_E3UW_B]) && !F[NEMO_F_E3UW_0])
    return fail(c, NEMO_ERR_UNBOUND, "dom_vvl_sf_swp: e3uw_0 must be bound with e3uw_n or e3uw_b");
  if ((F[NEMO_F_E3VW_N] || F[NEMO_F_E3VW_B]) && !F[NEMO_F_E3VW_0])
    return fail(c, NEMO_ERR_UNBOUND, "dom_vvl_sf_swp: e3vw_0 must be bound with e3vw_n or e3vw_b");
  if ((F[NEMO_F_E3UW_B] && !F[NEMO_F_E3U_B]) || (F[NEMO_F_E3VW_B] && !F[NEMO_F_E3V_B]))
    return fail(c, NEMO_ERR_UNBOUND, "dom_vvl_sf_swp: e3u_b, e3v_b must be bound with e3uw_b, e3vw_b");
  return c->prec == NEMO_PREC_FP64 ? run_vvl<double>(c, kt, VVL_SF_SWP) : run_vvl<float>(c, kt, VVL_SF_SWP);
}

// ---------------------------------------------------------------------- adjoint
static int adj_check(nemo_ctx* c, const char* cdtype, int* is_trc, const char* what) {
  if (c->prec != NEMO_PREC_FP64) return fail(c, NEMO_ERR_ARG, "%s: adjoints need an FP64 context", what);
  if (join_copies(c)) return NEMO_ERR_CUDA;
  if (cdtype) return check_cdtype(c, cdtype, is_trc);
  return NEMO_OK;
}

static int ensure_adj_work(nemo_ctx* c, int kjpt) {
  if (kjpt <= c->adj_kjpt) return NEMO_OK;
  const size_t bytes = (size_t)kjpt * c->n3 * c->nmem * sizeof(double);
  for (auto& p : c->adj_w) {
    cudaFree(p);
    p = nullptr;
  }
  for (auto& p : c->adj_w)
    if (cudaMalloc(&p, bytes) != cudaSuccess) return fail(c, NEMO_ERR_NOMEM, "adjoint work arrays (%zu bytes)", bytes);
  c->adj_kjpt = kjpt;
  return NEMO_OK;
}

int nemo_gpu_tra_adv_fct_adj(nemo_ctx* c, int kt, int kit000, const char* cdtype, double p2dt, const void* pun,
                             const void* pvn, const void* pwn, void* ptb_ad, void* ptn_ad, const void* pta_ad,
                             int kjpt, int kn_fct_h, int kn_fct_v) {
  (void)kt; (void)kit000; (void)p2dt;
  if (!c) return NEMO_ERR_ARG;
  int is_trc = 0;
  if (int s = adj_check(c, cdtype, &is_trc, "tra_adv_fct_adj")) return s;
  if (!pun || !pvn || !pwn || !ptb_ad || !ptn_ad || !pta_ad || kjpt < 1)
    return fail(c, NEMO_ERR_ARG, "tra_adv_fct_adj: bad argument");
  if ((kn_fct_h != 2 && kn_fct_h != 4) || (kn_fct_v != 2 && kn_fct_v != 4))
    return fail(c, NEMO_ERR_ARG, "tra_adv_fct_adj: kn_fct_h and kn_fct_v must be 2 or 4");
  if (kn_fct_v == 4 && c->nam.ln_isfcav)
    return fail(c, NEMO_ERR_UNSUPPORTED, "tra_adv_fct_adj: the compact vertical scheme without cavities");
  if (kn_fct_v == 4 && !c->fadj_w &&
      cudaMalloc(&c->fadj_w, 2 * (size_t)c->n3 * c->nmem * sizeof(double)) != cudaSuccess)
    return fail(c, NEMO_ERR_NOMEM, "tra_adv_fct_adj work arrays");
  if (!c->f[NEMO_F_FCT_TAPE])
    return fail(c, NEMO_ERR_UNBOUND, "tra_adv_fct_adj: the limiter tape NEMO_F_FCT_TAPE must be bound");
  FctAdj a{};
  a.pun = (const double*)pun; a.pvn = (const double*)pvn; a.pwn = (const double*)pwn;
  a.lam = (const double*)pta_ad; a.tape = (const double*)c->f[NEMO_F_FCT_TAPE];
  a.tb_ad = (double*)ptb_ad; a.tn_ad = (double*)ptn_ad;
  a.kjpt = kjpt; a.linssh = c->nam.ln_linssh;
  a.kh = kn_fct_h; a.kv = kn_fct_v;
  a.zwt = c->fadj_w; a.za = c->fadj_w ? c->fadj_w + (size_t)c->n3 * c->nmem : nullptr;
  cudaError_t e = launch_fct_adj(dom_now<double>(c), a, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "tra_adv_fct_adj launch");
  return NEMO_OK;
}

int nemo_gpu_tra_ldf_lap_adj(nemo_ctx* c, int kt, int kit000, const char* cdtype, const void* pahu, const void* pahv,
                             const void* pgu, const void* pgv, const void* pgui, const void* pgvi, void* ptb_ad,
                             const void* pta_ad, int kjpt, int kpass) {
  (void)kt; (void)kit000; (void)pgui; (void)pgvi;
  if (!c) return NEMO_ERR_ARG;
  int is_trc = 0;
  if (int s = adj_check(c, cdtype, &is_trc, "tra_ldf_lap_adj")) return s;
  if (!ptb_ad || !pta_ad || kjpt < 1 || (kpass != 1 && kpass != 2))
    return fail(c, NEMO_ERR_ARG, "tra_ldf_lap_adj: bad argument");
  LdfArgs<double> a = ldf_args<double>(c, pahu, pahv, pgu, pgv, nullptr, nullptr, nullptr, kjpt, kpass);
  LdfAdj b{};
  b.lam = (const double*)pta_ad; b.tb_ad = (double*)ptb_ad;
  cudaError_t e = launch_lap_adj(dom_now<double>(c), a, b, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "tra_ldf_lap_adj launch");
  return NEMO_OK;
}

int nemo_gpu_tra_ldf_iso_adj(nemo_ctx* c, int kt, int kit000, const char* cdtype, const void* pahu, const void* pahv,
                             const void* pgu, const void* pgv, const void* pgui, const void* pgvi, void* ptb_ad,
                             void* ptbb_ad, const void* pta_ad, int kjpt, int kpass) {
  (void)kt; (void)kit000; (void)pgui; (void)pgvi;
  if (!c) return NEMO_ERR_ARG;
  int is_trc = 0;
  if (int s = adj_check(c, cdtype, &is_trc, "tra_ldf_iso_adj")) return s;
  const nemo_namelist& nm = c->nam;
  if (!ptb_ad || !pta_ad || kjpt < 1 || (kpass != 1 && kpass != 2) || (kpass == 2 && !nm.ln_traldf_lap && !ptbb_ad))
    return fail(c, NEMO_ERR_ARG, "tra_ldf_iso_adj: bad argument");
  if (!c->f[NEMO_F_USLP] || !c->f[NEMO_F_VSLP] || !c->f[NEMO_F_WSLPI] || !c->f[NEMO_F_WSLPJ] ||
      !c->f[NEMO_F_AH_WSLP2] || !c->f[NEMO_F_AKZ])
    return fail(c, NEMO_ERR_UNBOUND, "tra_ldf_iso_adj: slopes, ah_wslp2 and akz must be bound");
  if (int s = ensure_adj_work(c, kjpt)) return s;
  LdfArgs<double> a = ldf_args<double>(c, pahu, pahv, pgu, pgv, nullptr, nullptr, nullptr, kjpt, kpass);
  a.uslp = (const double*)c->f[NEMO_F_USLP]; a.vslp = (const double*)c->f[NEMO_F_VSLP];
  a.wslpi = (const double*)c->f[NEMO_F_WSLPI]; a.wslpj = (const double*)c->f[NEMO_F_WSLPJ];
  a.ah_wslp2 = (double*)c->f[NEMO_F_AH_WSLP2]; a.akz = (double*)c->f[NEMO_F_AKZ];
  a.lap = nm.ln_traldf_lap; a.blp = nm.ln_traldf_blp; a.msc = nm.ln_traldf_msc;
  LdfAdj b{};
  b.lam = (const double*)pta_ad; b.tb_ad = (double*)ptb_ad; b.tbb_ad = (double*)ptbb_ad;
  b.G = (double*)c->adj_w[0]; b.dit = (double*)c->adj_w[1]; b.djt = (double*)c->adj_w[2]; b.dk = (double*)c->adj_w[3];
  cudaError_t e = launch_iso_adj(dom_now<double>(c), a, b, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "tra_ldf_iso_adj launch");
  return NEMO_OK;
}

int nemo_gpu_tra_zdf_imp_adj(nemo_ctx* c, int kt, int kit000, const char* cdtype, double p2dt, void* ptb_ad,
                             void* pta_ad, int kjpt) {
  (void)kt; (void)kit000;
  if (!c) return NEMO_ERR_ARG;
  int is_trc = 0;
  if (int s = adj_check(c, cdtype, &is_trc, "tra_zdf_imp_adj")) return s;
  if (!ptb_ad || !pta_ad || kjpt < 1) return fail(c, NEMO_ERR_ARG, "tra_zdf_imp_adj: bad argument");
  const nemo_namelist& nm = c->nam;
  ZdfArgs<double> a{};
  a.p2dt = p2dt; a.kjpt = kjpt;
  a.avt = (const double*)c->f[NEMO_F_AVT]; a.avs = (const double*)c->f[NEMO_F_AVS];
  a.ddm = nm.ln_zdfddm; a.is_trc = is_trc;
  if (!is_trc && !a.avt) return fail(c, NEMO_ERR_UNBOUND, "tra_zdf_imp_adj: avt must be bound");
  if ((is_trc || nm.ln_zdfddm) && !a.avs) return fail(c, NEMO_ERR_UNBOUND, "tra_zdf_imp_adj: avs must be bound");
  if (nm.ln_traldf_iso) {
    a.add = (const double*)c->f[nm.ln_traldf_msc ? NEMO_F_AKZ : NEMO_F_AH_WSLP2];
    if (!a.add) return fail(c, NEMO_ERR_UNBOUND, "tra_zdf_imp_adj: ah_wslp2/akz must be bound");
  }
  ZdfAdj b{(double*)pta_ad, (double*)ptb_ad};
  cudaError_t e = launch_zdf_adj(dom_now<double>(c), a, b, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "tra_zdf_imp_adj launch");
  return NEMO_OK;
}

int nemo_gpu_dyn_spg_ts_adj(nemo_ctx* c, int kt, const nemo_spg_adj* adj) {
  if (!c) return NEMO_ERR_ARG;
  if (c->prec != NEMO_PREC_FP64) return fail(c, NEMO_ERR_ARG, "dyn_spg_ts_adj: FP64 contexts only");
  if (!adj) return fail(c, NEMO_ERR_ARG, "dyn_spg_ts_adj: adj is NULL");
  void* const ptrs[] = {adj->ua, adj->va, adj->un, adj->vn, adj->ssha, adj->ua_b, adj->va_b, adj->un_adv, adj->vn_adv,
                        adj->ub2_b, adj->vb2_b, adj->un_bf, adj->vn_bf, adj->sshn, adj->un_b, adj->vn_b, adj->ub_b,
                        adj->vb_b};
  for (void* q : ptrs)
    if (!q) return fail(c, NEMO_ERR_ARG, "dyn_spg_ts_adj: null adjoint array");
  const nemo_namelist& nm = c->nam;
  if (!nm.ln_linssh || !nm.ln_bt_fw || !nm.ln_bt_av || nm.nvor_scheme == NEMO_VOR_ENT)
    return fail(c, NEMO_ERR_UNSUPPORTED,
                "dyn_spg_ts_adj: linear free surface with ln_bt_fw and ln_bt_av, vorticity ENE, ENS, EEN or MIX");
  if (!c->f[NEMO_F_RCDU_BOT]) return fail(c, NEMO_ERR_UNBOUND, "dyn_spg_ts_adj: rcdu_bot must be bound");
  if (c->icycle < 1 || (int)c->wgt1.size() < c->icycle)
    return fail(c, NEMO_ERR_STATE, "dyn_spg_ts_adj: run the forward dyn_spg_ts first (sub-step weights)");
  if (join_copies(c)) return NEMO_ERR_CUDA;
  const size_t n2m = (size_t)c->n2 * c->nmem;
  if (!c->spgadj_w && cudaMalloc(&c->spgadj_w, 18 * n2m * sizeof(double)) != cudaSuccess)
    return fail(c, NEMO_ERR_NOMEM, "dyn_spg_ts_adj work arrays");
  SpgAdjArgs a{};
  a.ua = (double*)adj->ua; a.va = (double*)adj->va; a.un = (double*)adj->un; a.vn = (double*)adj->vn;
  a.ssha = (double*)adj->ssha; a.ua_b = (double*)adj->ua_b; a.va_b = (double*)adj->va_b;
  a.un_adv = (double*)adj->un_adv; a.vn_adv = (double*)adj->vn_adv;
  a.ub2_b = (double*)adj->ub2_b; a.vb2_b = (double*)adj->vb2_b; a.un_bf = (double*)adj->un_bf;
  a.vn_bf = (double*)adj->vn_bf;
  a.sshn = (double*)adj->sshn; a.un_b = (double*)adj->un_b; a.vn_b = (double*)adj->vn_b;
  a.ub_b = (double*)adj->ub_b; a.vb_b = (double*)adj->vb_b;
  a.rcdu = (const double*)c->f[NEMO_F_RCDU_BOT];
  double* w = c->spgadj_w;
  double** work[] = {&a.X, &a.Y, &a.uab, &a.vab, &a.Au, &a.Aub, &a.Aubb, &a.Av, &a.Avb, &a.Avbb,
                     &a.Sn, &a.Sb, &a.Sbb, &a.Fu, &a.Fv, &a.gu, &a.gv, &a.zhd};
  for (int i = 0; i < 18; ++i) *work[i] = w + (size_t)i * n2m;
  const int euler = kt == nm.nit000 && nm.neuler == 0;
  a.euler = euler;
  a.r1_2dt_b = 1.0 / (euler ? nm.rn_rdt : 2.0 * nm.rn_rdt);
  a.atfp = nm.rn_atfp; a.rdtbt = c->rdtbt; a.grav = nm.grav; a.sl = nm.rn_scal_load;
  a.sc = nm.nvor_scheme;
  // the per-sub-step constants of the forward (dynspg_ts.F90:724-736, :904-931), ll_init
  std::vector<SpgAdjStep> steps(c->icycle);
  for (int jn = 1; jn <= c->icycle; ++jn) {
    SpgAdjStep& s = steps[jn - 1];
    s.w1 = c->wgt1[jn - 1]; s.w2 = c->wgt2[jn - 1];
    if (jn < 3) { s.zb1 = 1.0; s.zb2 = 0.0; s.zb3 = 0.0; }
    else { s.zb1 = 1.781105; s.zb2 = -1.06221; s.zb3 = 0.281105; }
    if (jn == 1) { s.za0 = 1.0; s.za1 = 0.0; s.za2 = 0.0; s.za3 = 0.0; }
    else if (jn == 2) { s.za0 = 1.0833333333333; s.za1 = -0.1666666666666; s.za2 = 0.0833333333333; s.za3 = 0.0; }
    else if (nm.rn_bt_alpha == 0.0) { s.za0 = 0.614; s.za1 = 0.285; s.za2 = 0.088; s.za3 = 0.013; }
    else {
      const double zepsilon = 0.00976186 - 0.13451357 * nm.rn_bt_alpha;
      const double zgamma = 0.08344500 - 0.51358400 * nm.rn_bt_alpha;
      s.za0 = 0.5 + zgamma + 2.0 * nm.rn_bt_alpha + 2.0 * zepsilon;
      s.za1 = 1.0 - s.za0 - zgamma - zepsilon;
      s.za2 = zgamma;
      s.za3 = zepsilon;
    }
  }
  cudaError_t e = launch_spg_adj(dom<double>(c), a, steps.data(), c->icycle, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "dyn_spg_ts_adj launch");
  return NEMO_OK;
}

int nemo_gpu_wzv_adj(nemo_ctx* c, int kt, void* un_ad, void* vn_ad, void* wn_ad) {
  (void)kt;
  if (!c) return NEMO_ERR_ARG;
  if (c->prec != NEMO_PREC_FP64) return fail(c, NEMO_ERR_ARG, "wzv_adj: FP64 contexts only");
  if (!un_ad || !vn_ad || !wn_ad) return fail(c, NEMO_ERR_ARG, "wzv_adj: null adjoint array");
  if (!c->nam.ln_linssh) return fail(c, NEMO_ERR_UNSUPPORTED, "wzv_adj: linear free surface only");
  if (join_copies(c)) return NEMO_ERR_CUDA;
  if (!c->wzvadj_w && cudaMalloc(&c->wzvadj_w, (size_t)c->n3 * c->nmem * sizeof(double)) != cudaSuccess)
    return fail(c, NEMO_ERR_NOMEM, "wzv_adj work array");
  cudaError_t e = launch_wzv_adj(dom<double>(c), (double*)un_ad, (double*)vn_ad, (double*)wn_ad, c->wzvadj_w,
                                 c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "wzv_adj launch");
  return NEMO_OK;
}

int nemo_gpu_dyn_nxt_adj(nemo_ctx* c, int kt, const nemo_nxt_adj* adj) {
  if (!c) return NEMO_ERR_ARG;
  if (c->prec != NEMO_PREC_FP64) return fail(c, NEMO_ERR_ARG, "dyn_nxt_adj: FP64 contexts only");
  if (!adj || !adj->ua || !adj->va || !adj->un || !adj->vn || !adj->ub || !adj->vb || !adj->un_b || !adj->vn_b ||
      !adj->ub_b || !adj->vb_b || !adj->ua_b || !adj->va_b)
    return fail(c, NEMO_ERR_ARG, "dyn_nxt_adj: null adjoint array");
  const nemo_namelist& nm = c->nam;
  if (!nm.ln_linssh || !nm.ln_bt_fw) return fail(c, NEMO_ERR_UNSUPPORTED, "dyn_nxt_adj: ln_linssh with ln_bt_fw only");
  if (join_copies(c)) return NEMO_ERR_CUDA;
  NxtAdjArgs a{};
  a.ua = (double*)adj->ua; a.va = (double*)adj->va; a.un = (double*)adj->un; a.vn = (double*)adj->vn;
  a.ub = (double*)adj->ub; a.vb = (double*)adj->vb;
  a.un_b = (double*)adj->un_b; a.vn_b = (double*)adj->vn_b; a.ub_b = (double*)adj->ub_b; a.vb_b = (double*)adj->vb_b;
  a.ua_b = (double*)adj->ua_b; a.va_b = (double*)adj->va_b;
  a.atfp = nm.rn_atfp;
  a.euler = nm.neuler == 0 && kt == nm.nit000;
  cudaError_t e = launch_dyn_nxt_adj(dom<double>(c), a, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "dyn_nxt_adj launch");
  return NEMO_OK;
}

int nemo_gpu_ssh_swp_adj(nemo_ctx* c, int kt, void* sshb_ad, void* sshn_ad, void* ssha_ad) {
  if (!c) return NEMO_ERR_ARG;
  if (c->prec != NEMO_PREC_FP64) return fail(c, NEMO_ERR_ARG, "ssh_swp_adj: FP64 contexts only");
  if (!sshb_ad || !sshn_ad || !ssha_ad) return fail(c, NEMO_ERR_ARG, "ssh_swp_adj: null adjoint array");
  const nemo_namelist& nm = c->nam;
  if (!nm.ln_linssh) return fail(c, NEMO_ERR_UNSUPPORTED, "ssh_swp_adj: linear free surface only");
  if (join_copies(c)) return NEMO_ERR_CUDA;
  cudaError_t e = launch_ssh_swp_adj(dom<double>(c), (double*)sshb_ad, (double*)sshn_ad, (double*)ssha_ad,
                                     nm.rn_atfp, nm.neuler == 0 && kt == nm.nit000, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "ssh_swp_adj launch");
  return NEMO_OK;
}

int nemo_gpu_tra_nxt_adj(nemo_ctx* c, int kt, void* tsb_ad, void* tsn_ad, void* tsa_ad) {
  if (!c) return NEMO_ERR_ARG;
  if (int s = adj_check(c, nullptr, nullptr, "tra_nxt_adj")) return s;
  if (!tsb_ad || !tsn_ad || !tsa_ad) return fail(c, NEMO_ERR_ARG, "tra_nxt_adj: null pointer");
  const nemo_namelist& nm = c->nam;
  if (!nm.ln_linssh) return fail(c, NEMO_ERR_ARG, "tra_nxt_adj: linear free surface only (ln_linssh)");
  const int euler = nm.neuler == 0 && kt == nm.nit000;
  cudaError_t e = launch_tra_nxt_adj(dom<double>(c), (double*)tsb_ad, (double*)tsn_ad, (double*)tsa_ad, nm.rn_atfp,
                                     euler, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "tra_nxt_adj launch");
  return NEMO_OK;
}

int nemo_gpu_dyn_spg_ts(nemo_ctx* c, int kt) {
  NvtxRange nvtx_range("dyn_spg_ts");
  if (!c) return NEMO_ERR_ARG;
  if (join_copies(c)) return NEMO_ERR_CUDA;
  return c->prec == NEMO_PREC_FP64 ? run_spg<double>(c, kt) : run_spg<float>(c, kt);
}

int nemo_gpu_lbc_lnk(nemo_ctx* c, const char* cdname, void* ptab, int nk, int nl, const char* cd_nat, double psgn,
                     double pval, int is_fp64) {
  NvtxRange nvtx_range("lbc_lnk");
  (void)cdname; (void)psgn;
  if (!c || !ptab || nk < 1 || nl < 1 || !cd_nat) return fail(c, NEMO_ERR_ARG, "lbc_lnk: bad argument");
  if (join_copies(c)) return NEMO_ERR_CUDA;
  const char n = cd_nat[0];
  if (n != 'T' && n != 'U' && n != 'V' && n != 'W' && n != 'F') return fail(c, NEMO_ERR_ARG, "lbc_lnk: bad grid nature");
  const long nslab = (long)nk * nl * c->nmem;
  cudaError_t e = is_fp64 ? launch_lbc<double>((double*)ptab, c->jpi, c->jpj, nslab, n == 'F', pval, c->stream)
                          : launch_lbc<float>((float*)ptab, c->jpi, c->jpj, nslab, n == 'F', (float)pval, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "lbc_lnk launch");
  return NEMO_OK;
}

int nemo_gpu_lbc_lnk_multi(nemo_ctx* c, const char* cdname, int kfld, void* const* ptabs, const int* nk,
                           const char* cd_nats, const double* psgns, double pval, int is_fp64) {
  if (!c || kfld < 1 || kfld > 9 || !ptabs || !nk || !cd_nats || !psgns) return fail(c, NEMO_ERR_ARG, "lbc_lnk_multi: bad argument");
  if (join_copies(c)) return NEMO_ERR_CUDA;
  for (int f = 0; f < kfld; ++f) {
    char nat[2] = {cd_nats[f], 0};
    int s = nemo_gpu_lbc_lnk(c, cdname, ptabs[f], nk[f], 1, nat, psgns[f], pval, is_fp64);
    if (s) return s;
  }
  return NEMO_OK;
}

int nemo_gpu_glob_sum(nemo_ctx* c, const char* cdname, const void* ptab, int nk, int is_fp64, double* out) {
  NvtxRange nvtx_range("glob_sum");
  (void)cdname;
  if (!c || !ptab || nk < 1 || !out) return fail(c, NEMO_ERR_ARG, "glob_sum: bad argument");
  if (join_copies(c)) return NEMO_ERR_CUDA;
  const double* tmi = c->prec == NEMO_PREC_FP64 ? c->dd.d.tmask_i.p : c->df.d.tmask_i.p;
  cudaError_t e = is_fp64 ? launch_globsum<double>((const double*)ptab, tmi, c->n2, nk, c->nmem, c->gs_part, c->gs_nblk,
                                                   c->gs_out, c->stream)
                          : launch_globsum<float>((const float*)ptab, tmi, c->n2, nk, c->nmem, c->gs_part, c->gs_nblk,
                                                  c->gs_out, c->stream);
  if (e != cudaSuccess) return cuda_fail(c, e, "glob_sum launch");
  CK(cudaMemcpyAsync(out, c->gs_out, (size_t)c->nmem * 8, cudaMemcpyDeviceToHost, c->stream), "glob_sum result");
  CK(cudaStreamSynchronize(c->stream), "glob_sum");
  return NEMO_OK;
}

static int stp_common(nemo_ctx* c, int kt, bool model) {
  if (!c) return NEMO_ERR_ARG;
  NvtxRange nvtx_range(model ? "stp" : "stp_hotpath");
  if (model)
    if (int s = model_fields(c, "stp_model")) return s;
  // host copies in flight: direct launches that wait per field (see run_hotpath);
  // otherwise the captured graph of the steady-state step
  if (!model && copies_pending(c) && !c->timing)
    return c->prec == NEMO_PREC_FP64 ? run_hotpath<double>(c, kt, true) : run_hotpath<float>(c, kt, true);
  if (join_copies(c)) return NEMO_ERR_CUDA;
  const nemo_namelist& nm = c->nam;
  if (model && nm.ln_usr)  // the forcing's scalars of this step, outside the graph
    if (int s = usr_put(c, kt)) return s;
  // class of kt: the Euler/leapfrog start steps differ in scalars and weights
  const int cls = kt == nm.nit000 ? 0 : (kt == nm.nit000 + 1 ? 1 : 2);
  const bool carry = !nm.ln_bt_av;  // ring rotation carries across calls: no replay
  const int key = cls + (model ? 10 : 0);
  if (cls == 2 && c->graphs_ok && !carry && !c->timing) {
    auto it = c->graphs.find(key);
    if (it != c->graphs.end()) {
      CK(cudaGraphLaunch(it->second, c->stream), "graph launch");
      return NEMO_OK;
    }
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      int s = c->prec == NEMO_PREC_FP64 ? run_hotpath<double>(c, kt, false, model)
                                        : run_hotpath<float>(c, kt, false, model);
      cudaError_t ee = cudaStreamEndCapture(c->stream, &g);
      cudaGraphExec_t ex = nullptr;
      if (s == NEMO_OK && ee == cudaSuccess && g && cudaGraphInstantiate(&ex, g, 0) == cudaSuccess) {
        cudaGraphDestroy(g);
        c->graphs[key] = ex;
        CK(cudaGraphLaunch(ex, c->stream), "graph launch");
        return NEMO_OK;
      }
      if (g) cudaGraphDestroy(g);
      cudaGetLastError();
      if (s != NEMO_OK) return s;
    }
    c->graphs_ok = false;  // capture unavailable: direct launches from now on
    cudaGetLastError();
  }
  return c->prec == NEMO_PREC_FP64 ? run_hotpath<double>(c, kt, false, model)
                                   : run_hotpath<float>(c, kt, false, model);
}

int nemo_gpu_stp_hotpath(nemo_ctx* c, int kt) { return stp_common(c, kt, false); }

int nemo_gpu_stp_model(nemo_ctx* c, int kt) { return stp_common(c, kt, true); }

// ------------------------------------------------------------------ autotuner
// The kernels of the hot path whose 32-wide block height the autotuner chooses
// (the TMA-staged and the persistent sub-step kernels have fixed tiles).
static const int kTunable[] = {NEMO_K_FCT_A, NEMO_K_FCT_B, NEMO_K_FCT_C, NEMO_K_ISO_FLUX, NEMO_K_ZDF_IMP,
                               NEMO_K_SPG_COR, NEMO_K_SPG_P1A, NEMO_K_SPG_P1B, NEMO_K_SPG_P3};

int nemo_gpu_autotune(nemo_ctx* c, int kt, int nrep) {
  if (!c) return NEMO_ERR_ARG;
  const nemo_namelist& nm = c->nam;
  if (nrep < 1) nrep = 3;
  if (kt <= nm.nit000 + 1) return fail(c, NEMO_ERR_ARG, "autotune: kt must be a steady-state step (> nit000 + 1)");
  if (!nm.ln_bt_av)
    return fail(c, NEMO_ERR_UNSUPPORTED, "autotune: the sub-step state carries across steps without ln_bt_av");
  if (join_copies(c)) return NEMO_ERR_CUDA;
  // every bound field the hot path writes, saved and put back before each trial step
  std::vector<std::pair<int, void*>> saved;
  auto bytes_of = [&](int id) {
    return field_numel(c, id) * c->nmem * (nemo_gpu_field_is_fp64(c, id) ? 8 : 4);
  };
  auto cleanup = [&]() {
    for (auto& p : saved) cudaFree(p.second);
  };
  for (int id = 0; id < NEMO_F_COUNT; ++id) {
    if (!c->f[id] || !(spg_writes(id) || id == NEMO_F_TSA || id == NEMO_F_AH_WSLP2 || id == NEMO_F_AKZ)) continue;
    void* p = nullptr;
    if (cudaMalloc(&p, bytes_of(id)) != cudaSuccess) {
      cleanup();
      return fail(c, NEMO_ERR_NOMEM, "autotune: copies of the written fields");
    }
    saved.push_back({id, p});
    CK(cudaMemcpyAsync(p, c->f[id], bytes_of(id), cudaMemcpyDeviceToDevice, c->stream), "autotune save");
  }
  auto restore = [&]() -> cudaError_t {
    for (auto& p : saved) {
      cudaError_t e = cudaMemcpyAsync(c->f[p.first], p.second, bytes_of(p.first), cudaMemcpyDeviceToDevice, c->stream);
      if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
  };
  const bool was_timing = c->timing;
  if (int s = nemo_gpu_set_timing(c, 1)) { cleanup(); return s; }
  double best[NEMO_K_COUNT];
  unsigned char pick[NEMO_K_COUNT] = {};
  for (double& b : best) b = 1e300;
  int st = NEMO_OK;
  for (int ty : {4, 2, 1}) {
    for (int id : kTunable) c->shape.ty[id] = (unsigned char)ty;
    for (int r = 0; r <= nrep && st == NEMO_OK; ++r) {
      if (r == 1) {  // the first step of each shape warms up
        for (double& t : c->kms) t = 0.0;
        for (int& n : c->kcnt) n = 0;
      }
      if (restore() != cudaSuccess) st = fail(c, NEMO_ERR_CUDA, "autotune restore");
      else st = c->prec == NEMO_PREC_FP64 ? run_hotpath<double>(c, kt, false) : run_hotpath<float>(c, kt, false);
    }
    if (st) break;
    for (int id : kTunable)
      if (c->kcnt[id] > 0 && c->kms[id] / c->kcnt[id] < best[id]) {
        best[id] = c->kms[id] / c->kcnt[id];
        pick[id] = (unsigned char)ty;
      }
  }
  for (int id : kTunable) c->shape.ty[id] = pick[id];
  if (restore() != cudaSuccess && st == NEMO_OK) st = fail(c, NEMO_ERR_CUDA, "autotune restore");
  cudaStreamSynchronize(c->stream);
  cleanup();
  nemo_gpu_set_timing(c, was_timing);
  for (auto& g : c->graphs) cudaGraphExecDestroy(g.second);  // recaptured with the chosen shapes
  c->graphs.clear();
  return st;
}

int nemo_gpu_set_launch_shape(nemo_ctx* c, const int* ty, int n) {
  if (!c || n < 0 || n > NEMO_K_COUNT || (n > 0 && !ty)) return fail(c, NEMO_ERR_ARG, "set_launch_shape: bad argument");
  bool tunable[NEMO_K_COUNT] = {};
  for (int id : kTunable) tunable[id] = true;
  for (int i = 0; i < n; ++i)
    if (!(ty[i] == 0 || ty[i] == 4 || (tunable[i] && (ty[i] == 1 || ty[i] == 2))))
      return fail(c, NEMO_ERR_ARG, "set_launch_shape: kernel %d cannot take block height %d", i, ty[i]);
  for (int i = 0; i < n; ++i) c->shape.ty[i] = (unsigned char)(ty[i] == 4 ? 0 : ty[i]);
  for (auto& g : c->graphs) cudaGraphExecDestroy(g.second);  // recaptured with the new shapes
  c->graphs.clear();
  return NEMO_OK;
}

int nemo_gpu_get_launch_shape(const nemo_ctx* c, int* ty, int n) {
  if (!c || n < 0 || (n > 0 && !ty)) return NEMO_ERR_ARG;
  for (int i = 0; i < n; ++i) ty[i] = i < NEMO_K_COUNT && c->shape.ty[i] ? c->shape.ty[i] : 4;
  return NEMO_OK;
}

int nemo_gpu_set_timing(nemo_ctx* c, int on) {
  if (!c) return NEMO_ERR_ARG;
  if (on && !c->tev[0]) {
    for (auto& e : c->tev) CK(cudaEventCreate(&e), "timing events");
    for (auto& e : c->kc.ev) CK(cudaEventCreate(&e), "timing events");
  }
  c->timing = on != 0;
  for (double& t : c->tms) t = 0.0;
  c->tcalls = 0;
  for (double& t : c->kms) t = 0.0;
  for (int& n : c->kcnt) n = 0;
  return NEMO_OK;
}

int nemo_gpu_get_kernel_timing(nemo_ctx* c, double* ms, int* launches, int n) {
  if (!c || n < 0 || (n > 0 && (!ms || !launches))) return NEMO_ERR_ARG;
  for (int i = 0; i < n; ++i) {
    ms[i] = i < NEMO_K_COUNT ? c->kms[i] : 0.0;
    launches[i] = i < NEMO_K_COUNT ? c->kcnt[i] : 0;
  }
  return NEMO_OK;
}

int nemo_gpu_get_timing(nemo_ctx* c, double* ms, int* ncalls) {
  if (!c || !ms) return NEMO_ERR_ARG;
  for (int i = 0; i < 4; ++i) ms[i] = c->tms[i];
  if (ncalls) *ncalls = c->tcalls;
  return NEMO_OK;
}

int nemo_gpu_set_fusion(nemo_ctx* c, int on) {
  if (!c) return NEMO_ERR_ARG;
  c->no_fusion = !on;
  for (auto& g : c->graphs) cudaGraphExecDestroy(g.second);
  c->graphs.clear();
  return NEMO_OK;
}

int nemo_gpu_set_fct_fused(nemo_ctx* c, int on) {
  if (!c) return NEMO_ERR_ARG;
  c->fct_fused = on != 0;
  for (auto& g : c->graphs) cudaGraphExecDestroy(g.second);
  c->graphs.clear();
  return NEMO_OK;
}

int nemo_gpu_set_tma(nemo_ctx* c, int on) {
  if (!c) return NEMO_ERR_ARG;
  c->no_tma = !on;
  for (auto& g : c->graphs) cudaGraphExecDestroy(g.second);
  c->graphs.clear();
  return NEMO_OK;
}

int nemo_gpu_set_spg_specialised(nemo_ctx* c, int on) {
  if (!c) return NEMO_ERR_ARG;
  c->no_p2_hot = !on;
  select_p2(c);
  for (auto& g : c->graphs) cudaGraphExecDestroy(g.second);
  c->graphs.clear();
  return c->p2_blocks < 1 ? fail(c, NEMO_ERR_CUDA, "set_spg_specialised: no launch shape") : NEMO_OK;
}

int nemo_gpu_set_tma_poll_limit(nemo_ctx* c, int max_polls) {
  if (!c || max_polls < 0) return fail(c, NEMO_ERR_ARG, "set_tma_poll_limit: bad argument");
  c->tma_polls = max_polls;
  for (auto& g : c->graphs) cudaGraphExecDestroy(g.second);
  c->graphs.clear();
  return NEMO_OK;
}

int nemo_gpu_set_barrier_limit(nemo_ctx* c, long long max_spins, int extra_arrivals) {
  if (!c || max_spins < 1 || extra_arrivals < 0) return fail(c, NEMO_ERR_ARG, "set_barrier_limit: bad argument");
  c->bar_spins = max_spins;
  c->bar_extra = extra_arrivals;
  for (auto& g : c->graphs) cudaGraphExecDestroy(g.second);
  c->graphs.clear();
  return NEMO_OK;
}

}  // extern "C"
