// Host side of the PT-TEMPO and process-tensor sweep C ABI.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/oqupy_gb300.h"
#include "capi_util.h"
#include "engine.h"

using namespace otb;

struct otb_pt {
  int n = 0;
  int precision = 0;
  int cap = 0;
  int grid = 0;
  int Dmax = 0;
  std::vector<PtDev> inst;
  std::vector<PtState> state;
  std::vector<int> order;
  DevBuf d_inst, d_state, d_dims, d_sites, d_infl, d_neg, d_caps, d_work, d_queue, d_order;
  long long wcap = 0;
  long long work_stride = 0;
};

namespace {

otb_status pt_check(otb_pt* h, int32_t inst) {
  if (!h) return set_error(OTB_ERR_INVALID_ARG, "null handle");
  if (inst < 0 || inst >= h->n) return set_error(OTB_ERR_INVALID_ARG, "instance index out of range");
  return OTB_OK;
}

otb_status pt_refresh(otb_pt* h, int32_t inst) {
  if (!check_cuda(cudaMemcpy(&h->state[inst], (PtState*)h->d_state.p + inst, sizeof(PtState),
                             cudaMemcpyDeviceToHost),
                  "read pt state"))
    return OTB_ERR_CUDA;
  return OTB_OK;
}

otb_status pt_dims(otb_pt* h, int32_t inst, std::vector<int2>& dims) {
  const PtDev& I = h->inst[inst];
  dims.resize(I.num_steps);
  if (!check_cuda(cudaMemcpy(dims.data(), (int2*)h->d_dims.p + I.dims_base,
                             sizeof(int2) * I.num_steps, cudaMemcpyDeviceToHost),
                  "read pt dims"))
    return OTB_ERR_CUDA;
  return OTB_OK;
}

}  // namespace

extern "C" otb_status otb_pt_create(const otb_pt_config* cfg, int32_t n, const otb_pt_instance* ins,
                                    otb_pt** out) {
  if (!cfg || !ins || !out || n <= 0) return set_error(OTB_ERR_INVALID_ARG, "bad arguments");
  *out = nullptr;
  if (cfg->precision != 0 && cfg->precision != 1)
    return set_error(OTB_ERR_INVALID_ARG, "precision must be 0 (complex128) or 1 (mixed)");
  if (cfg->chi_cap < 4 || cfg->chi_cap > 1152)
    return set_error(OTB_ERR_INVALID_ARG, "chi_cap must be in [4, 1152 / D]");
  std::unique_ptr<otb_pt> h(new otb_pt());
  h->n = n;
  if (!(cfg->qr_cut >= 0.0) || !(cfg->qr_cut < 1.0))
    return set_error(OTB_ERR_INVALID_ARG, "qr_cut must be in [0, 1)");
  h->precision = cfg->precision;
  h->cap = cfg->chi_cap;
  h->inst.resize(n);
  h->state.assign(n, PtState{});
  std::vector<double> infl, neg;
  long long site_total = 0, dims_total = 0, caps_total = 0;
  for (int i = 0; i < n; ++i) {
    const otb_pt_instance& s = ins[i];
    if (s.hs_dim < 1 || s.hs_dim > 3) return set_error(OTB_ERR_INVALID_ARG, "hs_dim must be 1..3");
    const int D = s.hs_dim * s.hs_dim;
    if (D > h->cap) return set_error(OTB_ERR_INVALID_ARG, "chi_cap must be >= D");
    if (D * h->cap > 1152) return set_error(OTB_ERR_INVALID_ARG, "chi_cap * D must be <= 1152");
    if (s.num_steps < 2) return set_error(OTB_ERR_INVALID_ARG, "num_steps must be >= 2");
    if (s.dkmax < 1) return set_error(OTB_ERR_INVALID_ARG, "dkmax must be >= 1");
    if (!(s.epsrel > 0.0) || !std::isfinite(s.epsrel))
      return set_error(OTB_ERR_INVALID_ARG, "epsrel must be positive and finite");
    if (!s.influences) return set_error(OTB_ERR_INVALID_ARG, "null influences");
    const int num_infl = std::min(s.num_steps, s.dkmax + 1);
    PtDev& I = h->inst[i];
    I.D = D;
    I.d = s.hs_dim;
    I.num_steps = s.num_steps;
    I.num_infl = num_infl;
    I.cap = h->cap;
    I.epsrel = s.epsrel;
    // A process tensor's truncation errors reach every step of the dynamics
    // built on it: the mixed form's default QR cut is 100x tighter than
    // TEMPO's (a bond-168 spin-boson process tensor: 2.7e-6 trace distance
    // at 1e-9, 1.2e-9 at 1e-11, for 14% more build time).
    I.qr_delta = cfg->qr_cut > 0.0 ? (float)cfg->qr_cut
                 : cfg->precision == 1 ? (float)std::fmin(1e-3 * s.epsrel, 1e-11) : 0.f;
    I.has_neg = s.neg_influences ? 1 : 0;
    I.site_base = site_total;
    site_total += (long long)s.num_steps * h->cap * D * h->cap;
    I.dims_base = dims_total;
    dims_total += s.num_steps;
    I.caps_base = caps_total;
    caps_total += (long long)(s.num_steps + 1) * h->cap;
    I.infl_base = (long long)infl.size() / 2;
    infl.insert(infl.end(), s.influences, s.influences + (size_t)num_infl * D * D * 2);
    I.neg_base = (long long)neg.size() / 2;
    if (s.neg_influences)
      neg.insert(neg.end(), s.neg_influences, s.neg_influences + (size_t)(s.num_steps + 1) * D * D * 2);
    h->Dmax = std::max(h->Dmax, D);
  }
  if (neg.empty()) neg.assign(2, 0.0);
  if (!h->d_sites.alloc((size_t)site_total * 16) || !h->d_dims.alloc((size_t)dims_total * sizeof(int2)) ||
      !h->d_caps.alloc((size_t)caps_total * 16) || !h->d_infl.alloc(infl.size() * sizeof(double)) ||
      !h->d_neg.alloc(neg.size() * sizeof(double)) || !h->d_inst.alloc(sizeof(PtDev) * n) ||
      !h->d_state.alloc(sizeof(PtState) * n) || !h->d_queue.alloc(sizeof(int)) ||
      !h->d_order.alloc(sizeof(int) * n))
    return OTB_ERR_OOM;
  if (!check_cuda(cudaMemset(h->d_dims.p, 0, (size_t)dims_total * sizeof(int2)), "memset") ||
      !check_cuda(cudaMemset(h->d_caps.p, 0, (size_t)caps_total * 16), "memset") ||
      !check_cuda(cudaMemcpy(h->d_infl.p, infl.data(), infl.size() * sizeof(double), cudaMemcpyHostToDevice), "upload") ||
      !check_cuda(cudaMemcpy(h->d_neg.p, neg.data(), neg.size() * sizeof(double), cudaMemcpyHostToDevice), "upload") ||
      !check_cuda(cudaMemcpy(h->d_inst.p, h->inst.data(), sizeof(PtDev) * n, cudaMemcpyHostToDevice), "upload") ||
      !check_cuda(cudaMemcpy(h->d_state.p, h->state.data(), sizeof(PtState) * n, cudaMemcpyHostToDevice), "upload"))
    return OTB_ERR_CUDA;
  h->order.resize(n);
  std::iota(h->order.begin(), h->order.end(), 0);
  std::stable_sort(h->order.begin(), h->order.end(), [&](int a, int b) {
    return (double)h->inst[a].num_steps * h->inst[a].num_infl > (double)h->inst[b].num_steps * h->inst[b].num_infl;
  });
  if (!check_cuda(cudaMemcpy(h->d_order.p, h->order.data(), sizeof(int) * n, cudaMemcpyHostToDevice), "upload"))
    return OTB_ERR_CUDA;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  h->grid = cfg->grid > 0 ? cfg->grid : std::max(1, std::min(n, 2 * std::max(sms, 1)));
  h->wcap = (long long)(h->cap * h->Dmax) * (h->cap * h->Dmax);
  h->work_stride = pt_work_bytes(h->wcap);
  if (!h->d_work.alloc((size_t)h->grid * h->work_stride)) return OTB_ERR_OOM;
  *out = h.release();
  return OTB_OK;
}

extern "C" void otb_pt_destroy(otb_pt* h) { delete h; }

extern "C" otb_status otb_pt_advance(otb_pt* h, int32_t nsteps, void* stream) {
  if (!h || nsteps < 0) return set_error(OTB_ERR_INVALID_ARG, "bad arguments");
  cudaStream_t s = (cudaStream_t)stream;
  if (!check_cuda(cudaMemsetAsync(h->d_queue.p, 0, sizeof(int), s), "reset queue")) return OTB_ERR_CUDA;
  PtLaunch L;
  L.n = h->n;
  L.inst = (const PtDev*)h->d_inst.p;
  L.state = (PtState*)h->d_state.p;
  L.dims = (int2*)h->d_dims.p;
  L.sites = h->d_sites.p;
  L.infl = (const double*)h->d_infl.p;
  L.neg = (const double*)h->d_neg.p;
  L.caps = (double*)h->d_caps.p;
  L.work = h->d_work.p;
  L.work_stride = h->work_stride;
  L.wcap = h->wcap;
  L.queue = (int*)h->d_queue.p;
  L.order = (const int*)h->d_order.p;
  L.nsteps = nsteps;
  L.smem_bytes = 0;
  if (!check_cuda(launch_pt(L, h->precision, h->grid, 256, s), "pt launch")) return OTB_ERR_CUDA;
  return OTB_OK;
}

extern "C" otb_status otb_pt_get_info(otb_pt* h, int32_t inst, otb_pt_info* info) {
  otb_status st = pt_check(h, inst);
  if (st) return st;
  if (!info) return set_error(OTB_ERR_INVALID_ARG, "null info");
  if ((st = pt_refresh(h, inst))) return st;
  const PtState& s = h->state[inst];
  info->step = s.step;
  info->status = s.status;
  info->num_steps = h->inst[inst].num_steps;
  info->splits = s.splits;
  info->sweeps64 = s.sweeps64;
  info->sweepsff = s.sweepsff;
  info->caps_done = s.caps_done;
  info->flops_alg = s.flops_alg;
  info->max_bond = 1;
  if (s.step > 0) {
    std::vector<int2> dims;
    if ((st = pt_dims(h, inst, dims))) return st;
    for (int k = 0; k < (int)dims.size(); ++k) info->max_bond = std::max(info->max_bond, dims[k].y);
  }
  return OTB_OK;
}

extern "C" otb_status otb_pt_bond_dims(otb_pt* h, int32_t inst, int32_t* out, int32_t cap) {
  otb_status st = pt_check(h, inst);
  if (st) return st;
  if (!out) return set_error(OTB_ERR_INVALID_ARG, "null output");
  std::vector<int2> dims;
  if ((st = pt_dims(h, inst, dims))) return st;
  const int N = h->inst[inst].num_steps;
  if (cap < N + 1) return set_error(OTB_ERR_INVALID_ARG, "output too small (need num_steps+1)");
  for (int k = 0; k < N; ++k) out[k] = dims[k].x;
  out[N] = dims[N - 1].y;
  return OTB_OK;
}

extern "C" otb_status otb_pt_get_tensor(otb_pt* h, int32_t inst, int32_t step, double* out,
                                        int64_t cap_elems, int32_t* dims_out) {
  otb_status st = pt_check(h, inst);
  if (st) return st;
  const PtDev& I = h->inst[inst];
  if (!out || !dims_out || step < 0 || step >= I.num_steps)
    return set_error(OTB_ERR_INVALID_ARG, "bad arguments");
  if ((st = pt_refresh(h, inst))) return st;
  if (h->state[inst].step < I.num_steps) return set_error(OTB_ERR_INVALID_ARG, "process tensor not complete");
  std::vector<int2> dims;
  if ((st = pt_dims(h, inst, dims))) return st;
  const int l = dims[step].x, r = dims[step].y, D = I.D;
  dims_out[0] = l;
  dims_out[1] = r;
  if (cap_elems < (int64_t)l * r * D) return set_error(OTB_ERR_INVALID_ARG, "output too small");
  std::vector<double> site((size_t)l * D * r * 2);
  const long long slot = (long long)I.cap * D * I.cap;
  if (!check_cuda(cudaMemcpy(site.data(), (double*)h->d_sites.p + 2 * (I.site_base + (long long)step * slot),
                             site.size() * sizeof(double), cudaMemcpyDeviceToHost),
                  "read site"))
    return OTB_ERR_CUDA;
  // [l][a][r] -> [l][r][a], times d (pt_tempo_backend.py:292-306)
  for (int ll = 0; ll < l; ++ll)
    for (int a = 0; a < D; ++a)
      for (int rr = 0; rr < r; ++rr) {
        const size_t src = 2 * (((size_t)ll * D + a) * r + rr);
        const size_t dst = 2 * (((size_t)ll * r + rr) * D + a);
        out[dst] = site[src] * I.d;
        out[dst + 1] = site[src + 1] * I.d;
      }
  return OTB_OK;
}

extern "C" otb_status otb_pt_get_cap(otb_pt* h, int32_t inst, int32_t step, double* out, int32_t cap,
                                     int32_t* count) {
  otb_status st = pt_check(h, inst);
  if (st) return st;
  const PtDev& I = h->inst[inst];
  if (!out || !count || step < 0 || step > I.num_steps) return set_error(OTB_ERR_INVALID_ARG, "bad arguments");
  if ((st = pt_refresh(h, inst))) return st;
  if (!h->state[inst].caps_done) return set_error(OTB_ERR_INVALID_ARG, "caps not computed yet");
  std::vector<int2> dims;
  if ((st = pt_dims(h, inst, dims))) return st;
  const int len = (step == I.num_steps) ? 1 : dims[step].x;
  *count = len;
  if (cap < len) return set_error(OTB_ERR_INVALID_ARG, "output too small");
  if (!check_cuda(cudaMemcpy(out, (double*)h->d_caps.p + 2 * (I.caps_base + (long long)step * I.cap),
                             sizeof(double) * 2 * len, cudaMemcpyDeviceToHost),
                  "read cap"))
    return OTB_ERR_CUDA;
  return OTB_OK;
}

// The sweep of nh systems over process tensor inst: ptab holds n_props
// propagator pairs (P1 then P2, D * D complex each), pidx (nh * num_steps,
// host) the pair of system h at step k.  Every index is checked here, on the
// host, before anything reaches the device.
static otb_status dyn_run_impl(otb_pt* h, int32_t inst, int32_t nh, const double* ptab, int32_t n_props,
                               const int32_t* pidx, const double* rho0, int32_t num_steps, double* out,
                               void* stream) {
  otb_status st = pt_check(h, inst);
  if (st) return st;
  const PtDev& I = h->inst[inst];
  if (!ptab || !rho0 || !out || nh < 1 || nh > 1024 || num_steps < 0 || num_steps > I.num_steps ||
      n_props < 1 || (num_steps > 0 && !pidx))
    return set_error(OTB_ERR_INVALID_ARG, "bad arguments");
  for (long long e = 0; e < (long long)nh * num_steps; ++e)
    if (pidx[e] < 0 || pidx[e] >= n_props)
      return set_error(OTB_ERR_INVALID_ARG, "propagator index out of range");
  if ((st = pt_refresh(h, inst))) return st;
  if (!h->state[inst].caps_done) return set_error(OTB_ERR_INVALID_ARG, "process tensor not complete");
  std::vector<int2> dims;
  if ((st = pt_dims(h, inst, dims))) return st;
  const int D = I.D;
  DevBuf dtab, didx, drho, dv0, dv1, dout;
  const size_t tb = (size_t)n_props * 2 * D * D * 16, vb = (size_t)nh * I.cap * D * 16;
  const size_t ib = (size_t)nh * std::max(num_steps, 1) * sizeof(int32_t);
  const size_t ob = (size_t)(num_steps + 1) * nh * D * 16;
  const int max_chunks = (I.cap + 31) / 32;
  DevBuf dpart, dcnt;
  if (!dtab.alloc(tb) || !didx.alloc(ib) || !drho.alloc((size_t)nh * D * 16) || !dv0.alloc(vb) ||
      !dv1.alloc(vb) || !dout.alloc(ob) || !dpart.alloc((size_t)nh * max_chunks * D * 16) ||
      !dcnt.alloc((size_t)nh * sizeof(unsigned int)))
    return OTB_ERR_OOM;
  cudaStream_t s = (cudaStream_t)stream;
  if (!check_cuda(cudaMemcpyAsync(dtab.p, ptab, tb, cudaMemcpyHostToDevice, s), "upload") ||
      (num_steps > 0 &&
       !check_cuda(cudaMemcpyAsync(didx.p, pidx, (size_t)nh * num_steps * sizeof(int32_t),
                                   cudaMemcpyHostToDevice, s), "upload")) ||
      !check_cuda(cudaMemcpyAsync(drho.p, rho0, (size_t)nh * D * 16, cudaMemcpyHostToDevice, s), "upload") ||
      !check_cuda(cudaMemsetAsync(dout.p, 0, ob, s), "memset") ||
      !check_cuda(cudaMemsetAsync(dv0.p, 0, vb, s), "memset") ||
      !check_cuda(cudaMemsetAsync(dcnt.p, 0, (size_t)nh * sizeof(unsigned int), s), "memset"))
    return OTB_ERR_CUDA;
  DynLaunch L;
  L.nh = nh;
  L.D = D;
  L.d = I.d;
  L.sites = (const double*)h->d_sites.p + 2 * I.site_base;
  L.slot_elems = (long long)I.cap * D * I.cap;
  L.dims = (const int2*)h->d_dims.p + I.dims_base;
  L.caps = (const double*)h->d_caps.p + 2 * I.caps_base;
  L.cap = I.cap;
  L.ptab = (const double*)dtab.p;
  L.pidx = (const int*)didx.p;
  L.pidx_stride = num_steps;
  L.vcur = (double*)dv0.p;
  L.vnext = (double*)dv1.p;
  L.out = (double*)dout.p;
  L.partial = (double*)dpart.p;
  L.counter = (unsigned int*)dcnt.p;
  L.max_chunks = max_chunks;
  L.k = 0;
  L.fwd_hist = nullptr;
  L.back_hist = nullptr;
  L.deriv = nullptr;
  L.hist_steps = 0;
  if (!check_cuda(launch_dyn_init(L, (const double*)drho.p, s), "dyn init")) return OTB_ERR_CUDA;
  // the whole sweep as one CUDA graph: one kernel node per step
  cudaStream_t cs;
  if (!check_cuda(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking), "stream")) return OTB_ERR_CUDA;
  cudaEvent_t ready;
  cudaEventCreateWithFlags(&ready, cudaEventDisableTiming);
  cudaEventRecord(ready, s);
  cudaStreamWaitEvent(cs, ready, 0);
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  bool ok = check_cuda(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal), "capture");
  for (int k = 0; ok && k < num_steps; ++k) {
    DynLaunch Lk = L;
    Lk.k = k;
    Lk.vcur = (k % 2 == 0) ? (double*)dv0.p : (double*)dv1.p;
    Lk.vnext = (k % 2 == 0) ? (double*)dv1.p : (double*)dv0.p;
    ok = check_cuda(launch_dyn_step(Lk, dims[k].y, cs), "dyn step");
  }
  cudaError_t ce = cudaStreamEndCapture(cs, &graph);
  ok = ok && check_cuda(ce, "end capture");
  if (ok) ok = check_cuda(cudaGraphInstantiate(&exec, graph, 0), "instantiate");
  if (ok) ok = check_cuda(cudaGraphLaunch(exec, cs), "graph launch");
  if (ok) {
    cudaEventRecord(ready, cs);
    cudaStreamWaitEvent(s, ready, 0);
    ok = check_cuda(cudaMemcpyAsync(out, dout.p, ob, cudaMemcpyDeviceToHost, s), "download") &&
         check_cuda(cudaStreamSynchronize(s), "sync");
  }
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  cudaEventDestroy(ready);
  cudaStreamDestroy(cs);
  return ok ? OTB_OK : OTB_ERR_CUDA;
}

// A sweep advanced one step per call, for callers that choose each step's
// propagators from the states so far (compute_dynamics_with_field,
// system_dynamics.py:184-476): the device keeps the states with their bond
// legs between calls.  The process tensor must outlive the session.
struct otb_dyn_session {
  otb_pt* pt = nullptr;
  int inst = 0;
  int nh = 0;
  int k = 0;            // steps done
  int num_steps = 0;    // the process tensor's length
  std::vector<int2> dims;
  DevBuf dtab, didx, dv0, dv1, dout, dpart, dcnt;
};

extern "C" otb_status otb_dyn_session_create(otb_pt* h, int32_t inst, int32_t nh, const double* rho0,
                                             otb_dyn_session** out) {
  if (!out) return set_error(OTB_ERR_INVALID_ARG, "null output");
  *out = nullptr;
  otb_status st = pt_check(h, inst);
  if (st) return st;
  if (!rho0 || nh < 1 || nh > 1024) return set_error(OTB_ERR_INVALID_ARG, "bad arguments");
  if ((st = pt_refresh(h, inst))) return st;
  if (!h->state[inst].caps_done) return set_error(OTB_ERR_INVALID_ARG, "process tensor not complete");
  std::unique_ptr<otb_dyn_session> ss(new otb_dyn_session());
  ss->pt = h;
  ss->inst = inst;
  ss->nh = nh;
  const PtDev& I = h->inst[inst];
  ss->num_steps = I.num_steps;
  if ((st = pt_dims(h, inst, ss->dims))) return st;
  const int D = I.D;
  const size_t vb = (size_t)nh * I.cap * D * 16;
  const size_t ob = (size_t)(I.num_steps + 1) * nh * D * 16;
  const int max_chunks = (I.cap + 31) / 32;
  if (!ss->dtab.alloc((size_t)nh * 2 * D * D * 16) || !ss->didx.alloc((size_t)nh * I.num_steps * sizeof(int32_t)) ||
      !ss->dv0.alloc(vb) || !ss->dv1.alloc(vb) || !ss->dout.alloc(ob) ||
      !ss->dpart.alloc((size_t)nh * max_chunks * D * 16) || !ss->dcnt.alloc((size_t)nh * sizeof(unsigned int)))
    return OTB_ERR_OOM;
  // system h always uses pair h of the table, which every step replaces
  std::vector<int32_t> idx((size_t)nh * I.num_steps);
  for (int i = 0; i < nh; ++i)
    for (int k = 0; k < I.num_steps; ++k) idx[(size_t)i * I.num_steps + k] = i;
  DevBuf drho;
  if (!drho.alloc((size_t)nh * D * 16)) return OTB_ERR_OOM;
  if (!check_cuda(cudaMemcpy(ss->didx.p, idx.data(), idx.size() * sizeof(int32_t), cudaMemcpyHostToDevice),
                  "upload") ||
      !check_cuda(cudaMemcpy(drho.p, rho0, (size_t)nh * D * 16, cudaMemcpyHostToDevice), "upload") ||
      !check_cuda(cudaMemset(ss->dout.p, 0, ob), "memset") || !check_cuda(cudaMemset(ss->dv0.p, 0, vb), "memset") ||
      !check_cuda(cudaMemset(ss->dcnt.p, 0, (size_t)nh * sizeof(unsigned int)), "memset"))
    return OTB_ERR_CUDA;
  DynLaunch L{};
  L.nh = nh;
  L.D = D;
  L.d = I.d;
  L.caps = (const double*)h->d_caps.p + 2 * I.caps_base;
  L.vcur = (double*)ss->dv0.p;
  L.out = (double*)ss->dout.p;
  if (!check_cuda(launch_dyn_init(L, (const double*)drho.p, 0), "dyn init") ||
      !check_cuda(cudaDeviceSynchronize(), "sync"))
    return OTB_ERR_CUDA;
  *out = ss.release();
  return OTB_OK;
}

extern "C" otb_status otb_dyn_session_step(otb_dyn_session* ss, const double* props, double* state_out,
                                           void* stream) {
  if (!ss || !props || !state_out) return set_error(OTB_ERR_INVALID_ARG, "bad arguments");
  if (ss->k >= ss->num_steps) return set_error(OTB_ERR_INVALID_ARG, "the process tensor has no further step");
  otb_pt* h = ss->pt;
  const PtDev& I = h->inst[ss->inst];
  const int D = I.D, nh = ss->nh, k = ss->k;
  cudaStream_t s = (cudaStream_t)stream;
  if (!check_cuda(cudaMemcpyAsync(ss->dtab.p, props, (size_t)nh * 2 * D * D * 16, cudaMemcpyHostToDevice, s),
                  "upload"))
    return OTB_ERR_CUDA;
  DynLaunch L{};
  L.nh = nh;
  L.D = D;
  L.d = I.d;
  L.sites = (const double*)h->d_sites.p + 2 * I.site_base;
  L.slot_elems = (long long)I.cap * D * I.cap;
  L.dims = (const int2*)h->d_dims.p + I.dims_base;
  L.caps = (const double*)h->d_caps.p + 2 * I.caps_base;
  L.cap = I.cap;
  L.ptab = (const double*)ss->dtab.p;
  L.pidx = (const int*)ss->didx.p;
  L.pidx_stride = ss->num_steps;
  L.vcur = (k % 2 == 0) ? (double*)ss->dv0.p : (double*)ss->dv1.p;
  L.vnext = (k % 2 == 0) ? (double*)ss->dv1.p : (double*)ss->dv0.p;
  L.out = (double*)ss->dout.p;
  L.partial = (double*)ss->dpart.p;
  L.counter = (unsigned int*)ss->dcnt.p;
  L.max_chunks = (I.cap + 31) / 32;
  L.k = k;
  if (!check_cuda(launch_dyn_step(L, ss->dims[k].y, s), "dyn step")) return OTB_ERR_CUDA;
  const size_t sb = (size_t)nh * D * 16;
  if (!check_cuda(cudaMemcpyAsync(state_out, (char*)ss->dout.p + (size_t)(k + 1) * sb, sb,
                                  cudaMemcpyDeviceToHost, s),
                  "download") ||
      !check_cuda(cudaStreamSynchronize(s), "sync"))
    return OTB_ERR_CUDA;
  ss->k = k + 1;
  return OTB_OK;
}

extern "C" otb_status otb_dyn_session_state(otb_dyn_session* ss, int32_t step, double* state_out) {
  if (!ss || !state_out || step < 0 || step > ss->k) return set_error(OTB_ERR_INVALID_ARG, "bad arguments");
  const size_t sb = (size_t)ss->nh * ss->pt->inst[ss->inst].D * 16;
  if (!check_cuda(cudaMemcpy(state_out, (char*)ss->dout.p + (size_t)step * sb, sb, cudaMemcpyDeviceToHost),
                  "download"))
    return OTB_ERR_CUDA;
  return OTB_OK;
}

extern "C" void otb_dyn_session_destroy(otb_dyn_session* ss) { delete ss; }

extern "C" otb_status otb_dyn_gradient(otb_pt* h, int32_t inst, int32_t nh, const double* props,
                                       int32_t n_props, const int32_t* prop_index, const double* rho0,
                                       const double* target, int32_t num_steps, double* out_states,
                                       double* out_cores, void* stream) {
  otb_status st = pt_check(h, inst);
  if (st) return st;
  const PtDev& I = h->inst[inst];
  if (!props || !prop_index || !rho0 || !target || !out_states || !out_cores || nh < 1 || nh > 1024 ||
      num_steps < 1 || num_steps > I.num_steps || n_props < 1)
    return set_error(OTB_ERR_INVALID_ARG, "bad arguments");
  for (long long e = 0; e < (long long)nh * num_steps; ++e)
    if (prop_index[e] < 0 || prop_index[e] >= n_props)
      return set_error(OTB_ERR_INVALID_ARG, "propagator index out of range");
  if ((st = pt_refresh(h, inst))) return st;
  if (!h->state[inst].caps_done) return set_error(OTB_ERR_INVALID_ARG, "process tensor not complete");
  std::vector<int2> dims;
  if ((st = pt_dims(h, inst, dims))) return st;
  // the target carries no bond: the sweep must end where the process tensor's bond closes
  if (dims[num_steps - 1].y != 1)
    return set_error(OTB_ERR_INVALID_ARG, "gradient needs num_steps = the process tensor's length (closed bond)");
  int max_r = 1;
  for (int k = 0; k < num_steps; ++k) max_r = std::max(max_r, std::max(dims[k].x, dims[k].y));
  const int D = I.D;
  const size_t tb = (size_t)n_props * 2 * D * D * 16, vb = (size_t)nh * I.cap * D * 16;
  const size_t ib = (size_t)nh * num_steps * sizeof(int32_t);
  const size_t ob = (size_t)(num_steps + 1) * nh * D * 16;
  const size_t fb = (size_t)nh * num_steps * I.cap * D * 16;
  const size_t bb = (size_t)nh * (num_steps + 1) * I.cap * D * 16;
  const size_t cb = (size_t)nh * num_steps * D * D * D * 16;
  const int max_chunks = (I.cap + 31) / 32;
  DevBuf dtab, didx, drho, dtgt, dv0, dv1, dout, dpart, dcnt, dfwd, dback, dcore;
  if (!dtab.alloc(tb) || !didx.alloc(ib) || !drho.alloc((size_t)nh * D * 16) ||
      !dtgt.alloc((size_t)nh * D * 16) || !dv0.alloc(vb) || !dv1.alloc(vb) || !dout.alloc(ob) ||
      !dpart.alloc((size_t)nh * max_chunks * D * 16) || !dcnt.alloc((size_t)nh * sizeof(unsigned int)) ||
      !dfwd.alloc(fb) || !dback.alloc(bb) || !dcore.alloc(cb))
    return OTB_ERR_OOM;
  cudaStream_t s = (cudaStream_t)stream;
  if (!check_cuda(cudaMemcpyAsync(dtab.p, props, tb, cudaMemcpyHostToDevice, s), "upload") ||
      !check_cuda(cudaMemcpyAsync(didx.p, prop_index, ib, cudaMemcpyHostToDevice, s), "upload") ||
      !check_cuda(cudaMemcpyAsync(drho.p, rho0, (size_t)nh * D * 16, cudaMemcpyHostToDevice, s), "upload") ||
      !check_cuda(cudaMemcpyAsync(dtgt.p, target, (size_t)nh * D * 16, cudaMemcpyHostToDevice, s), "upload") ||
      !check_cuda(cudaMemsetAsync(dout.p, 0, ob, s), "memset") ||
      !check_cuda(cudaMemsetAsync(dv0.p, 0, vb, s), "memset") ||
      !check_cuda(cudaMemsetAsync(dfwd.p, 0, fb, s), "memset") ||
      !check_cuda(cudaMemsetAsync(dback.p, 0, bb, s), "memset") ||
      !check_cuda(cudaMemsetAsync(dcnt.p, 0, (size_t)nh * sizeof(unsigned int), s), "memset"))
    return OTB_ERR_CUDA;
  DynLaunch L;
  L.nh = nh;
  L.D = D;
  L.d = I.d;
  L.sites = (const double*)h->d_sites.p + 2 * I.site_base;
  L.slot_elems = (long long)I.cap * D * I.cap;
  L.dims = (const int2*)h->d_dims.p + I.dims_base;
  L.caps = (const double*)h->d_caps.p + 2 * I.caps_base;
  L.cap = I.cap;
  L.ptab = (const double*)dtab.p;
  L.pidx = (const int*)didx.p;
  L.pidx_stride = num_steps;
  L.vcur = (double*)dv0.p;
  L.vnext = (double*)dv1.p;
  L.out = (double*)dout.p;
  L.partial = (double*)dpart.p;
  L.counter = (unsigned int*)dcnt.p;
  L.max_chunks = max_chunks;
  L.k = 0;
  L.fwd_hist = (double*)dfwd.p;
  L.back_hist = (double*)dback.p;
  L.deriv = (double*)dcore.p;
  L.hist_steps = num_steps;
  if (!check_cuda(launch_dyn_init(L, (const double*)drho.p, s), "dyn init")) return OTB_ERR_CUDA;
  for (int k = 0; k < num_steps; ++k) {
    DynLaunch Lk = L;
    Lk.k = k;
    Lk.vcur = (k % 2 == 0) ? (double*)dv0.p : (double*)dv1.p;
    Lk.vnext = (k % 2 == 0) ? (double*)dv1.p : (double*)dv0.p;
    if (!check_cuda(launch_dyn_step(Lk, dims[k].y, s), "forward step")) return OTB_ERR_CUDA;
  }
  if (!check_cuda(launch_dyn_back_init(L, (const double*)dtgt.p, s), "adjoint init")) return OTB_ERR_CUDA;
  for (int k = num_steps - 1; k >= 1; --k) {
    DynLaunch Lk = L;
    Lk.k = k;
    if (!check_cuda(launch_dyn_back_step(Lk, dims[k].x, dims[k].y, s), "adjoint step")) return OTB_ERR_CUDA;
  }
  if (!check_cuda(launch_dyn_deriv(L, num_steps, max_r, s), "derivative cores")) return OTB_ERR_CUDA;
  if (!check_cuda(cudaMemcpyAsync(out_states, dout.p, ob, cudaMemcpyDeviceToHost, s), "download") ||
      !check_cuda(cudaMemcpyAsync(out_cores, dcore.p, cb, cudaMemcpyDeviceToHost, s), "download") ||
      !check_cuda(cudaStreamSynchronize(s), "sync"))
    return OTB_ERR_CUDA;
  return OTB_OK;
}

extern "C" otb_status otb_dyn_run(otb_pt* h, int32_t inst, int32_t nh, const double* p1, const double* p2,
                                  const double* rho0, int32_t num_steps, double* out, void* stream) {
  otb_status st = pt_check(h, inst);
  if (st) return st;
  if (!p1 || !p2 || nh < 1 || nh > 1024 || num_steps < 0)
    return set_error(OTB_ERR_INVALID_ARG, "bad arguments");
  const int D = h->inst[inst].D;
  const size_t dd = (size_t)2 * D * D;   // doubles of one D x D complex matrix
  std::vector<double> tab((size_t)nh * 2 * dd);
  for (int i = 0; i < nh; ++i) {
    std::copy(p1 + i * dd, p1 + (i + 1) * dd, tab.begin() + (size_t)i * 2 * dd);
    std::copy(p2 + i * dd, p2 + (i + 1) * dd, tab.begin() + (size_t)i * 2 * dd + dd);
  }
  std::vector<int32_t> idx((size_t)nh * std::max(num_steps, 1));
  for (int i = 0; i < nh; ++i)
    for (int k = 0; k < num_steps; ++k) idx[(size_t)i * num_steps + k] = i;
  return dyn_run_impl(h, inst, nh, tab.data(), nh, idx.data(), rho0, num_steps, out, stream);
}

extern "C" otb_status otb_dyn_run_steps(otb_pt* h, int32_t inst, int32_t nh, const double* props,
                                        int32_t n_props, const int32_t* prop_index, const double* rho0,
                                        int32_t num_steps, double* out, void* stream) {
  return dyn_run_impl(h, inst, nh, props, n_props, prop_index, rho0, num_steps, out, stream);
}
