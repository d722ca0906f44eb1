// Host side of the batched TEMPO C ABI (include/oqupy_gb300.h).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/oqupy_gb300.h"
#include "capi_util.h"
#include "engine.h"

using namespace otb;

struct otb_tempo {
  int n = 0;
  int precision = 0;
  int cap = 0;
  int out_cap = 0;
  int grid = 0;
  int grid_alloc = 0;   // CTAs the per-CTA workspace is allocated for
  int sms = 0;
  int block = 256;
  int smem_bytes = 0;
  int Dmax = 0;
  size_t elem = 16;  // bytes per site element (complex128 in both forms)
  std::vector<InstDev> inst;
  std::vector<InstState> state;  // host shadow (refreshed on demand)
  std::vector<int> order;
  std::vector<std::vector<double>> infl_host;  // per instance, growing
  DevBuf d_inst, d_state, d_dims, d_sites, d_infl, d_props, d_out, d_work, d_queue, d_order;
  long long wcap = 0;
  long long work_stride = 0;
  long long props_elems = 0;  // complex elements in d_props
};

namespace {

long long slot_elems(const otb_tempo* h, int D) { return (long long)h->cap * D * h->cap; }

// (Re)build the site arena and dims for the given per-instance slot counts,
// copying existing rings (linearised from their heads) when `keep` is set.
otb_status layout_sites(otb_tempo* h, const std::vector<int>& nslots, bool keep) {
  long long site_total = 0, dims_total = 0;
  std::vector<long long> sb(h->n), db(h->n);
  for (int i = 0; i < h->n; ++i) {
    sb[i] = site_total;
    db[i] = dims_total;
    site_total += (long long)nslots[i] * slot_elems(h, h->inst[i].D);
    dims_total += nslots[i];
  }
  DevBuf sites, dims;
  if (!sites.alloc((size_t)site_total * h->elem)) return OTB_ERR_OOM;
  if (!dims.alloc((size_t)dims_total * sizeof(int2))) return OTB_ERR_OOM;
  if (!check_cuda(cudaMemset(dims.p, 0, (size_t)dims_total * sizeof(int2)), "memset dims"))
    return OTB_ERR_CUDA;
  if (keep) {
    if (!check_cuda(cudaMemcpy(h->state.data(), h->d_state.p, sizeof(InstState) * h->n,
                               cudaMemcpyDeviceToHost),
                    "read state"))
      return OTB_ERR_CUDA;
    for (int i = 0; i < h->n; ++i) {
      const InstDev& I = h->inst[i];
      InstState& st = h->state[i];
      const long long se = slot_elems(h, I.D);
      for (int k = 0; k < st.nsites; ++k) {
        const int from = (st.head + k) % I.nslots;
        if (!check_cuda(cudaMemcpy((char*)sites.p + (sb[i] + (long long)k * se) * h->elem,
                                   (char*)h->d_sites.p + (I.site_base + (long long)from * se) * h->elem,
                                   (size_t)se * h->elem, cudaMemcpyDeviceToDevice),
                        "copy site"))
          return OTB_ERR_CUDA;
        if (!check_cuda(cudaMemcpy((int2*)dims.p + db[i] + k,
                                   (int2*)h->d_dims.p + I.dims_base + from, sizeof(int2),
                                   cudaMemcpyDeviceToDevice),
                        "copy dims"))
          return OTB_ERR_CUDA;
      }
      st.head = 0;
    }
    if (!check_cuda(cudaMemcpy(h->d_state.p, h->state.data(), sizeof(InstState) * h->n,
                               cudaMemcpyHostToDevice),
                    "write state"))
      return OTB_ERR_CUDA;
  }
  for (int i = 0; i < h->n; ++i) {
    h->inst[i].site_base = sb[i];
    h->inst[i].dims_base = db[i];
    h->inst[i].nslots = nslots[i];
  }
  h->d_sites = std::move(sites);
  h->d_dims = std::move(dims);
  return OTB_OK;
}

otb_status upload_infl(otb_tempo* h) {
  long long total = 0;
  for (int i = 0; i < h->n; ++i) total += (long long)h->infl_host[i].size() / 2;
  std::vector<double> flat;
  flat.reserve((size_t)total * 2);
  for (int i = 0; i < h->n; ++i) {
    h->inst[i].infl_base = (long long)flat.size() / 2;
    const int D = h->inst[i].D;
    h->inst[i].ninfl = (int)(h->infl_host[i].size() / (2 * D * D));
    flat.insert(flat.end(), h->infl_host[i].begin(), h->infl_host[i].end());
  }
  DevBuf d;
  if (!d.alloc(flat.size() * sizeof(double))) return OTB_ERR_OOM;
  if (!check_cuda(cudaMemcpy(d.p, flat.data(), flat.size() * sizeof(double), cudaMemcpyHostToDevice),
                  "upload influences"))
    return OTB_ERR_CUDA;
  h->d_infl = std::move(d);
  return OTB_OK;
}

otb_status upload_inst(otb_tempo* h) {
  if (!check_cuda(cudaMemcpy(h->d_inst.p, h->inst.data(), sizeof(InstDev) * h->n,
                             cudaMemcpyHostToDevice),
                  "upload instances"))
    return OTB_ERR_CUDA;
  return OTB_OK;
}

otb_status check_inst(otb_tempo* h, int32_t inst) {
  if (!h) return set_error(OTB_ERR_INVALID_ARG, "null handle");
  if (inst < 0 || inst >= h->n) return set_error(OTB_ERR_INVALID_ARG, "instance index out of range");
  return OTB_OK;
}

}  // namespace

extern "C" otb_status otb_tempo_create(const otb_tempo_config* cfg, int32_t n,
                                       const otb_tempo_instance* ins, otb_tempo** out) {
  if (!cfg || !ins || !out || n <= 0) return set_error(OTB_ERR_INVALID_ARG, "bad arguments");
  *out = nullptr;
  if (cfg->precision != OTB_PRECISION_COMPLEX128 && cfg->precision != OTB_PRECISION_MIXED)
    return set_error(OTB_ERR_INVALID_ARG, "precision must be 0 (complex128) or 1 (mixed)");
  if (cfg->chi_cap < 4 || cfg->chi_cap > 1152)
    return set_error(OTB_ERR_INVALID_ARG, "chi_cap must be in [4, 1152 / D]");
  if (cfg->out_cap < 2) return set_error(OTB_ERR_INVALID_ARG, "out_cap must be >= 2");
  if (cfg->block != 0 && (cfg->block < 64 || cfg->block > 512 || cfg->block % 32 != 0))
    return set_error(OTB_ERR_INVALID_ARG, "block must be 0 or a multiple of 32 in [64, 512]");
  if (cfg->smem_kb < 0 || cfg->smem_kb > 200)
    return set_error(OTB_ERR_INVALID_ARG, "smem_kb must be in [0, 200]");
  if (!(cfg->qr_cut >= 0.0) || !(cfg->qr_cut < 1.0))
    return set_error(OTB_ERR_INVALID_ARG, "qr_cut must be in [0, 1)");
  std::unique_ptr<otb_tempo> h(new otb_tempo());
  h->block = cfg->block > 0 ? cfg->block : 256;
  h->smem_bytes = cfg->smem_kb * 1024;
  h->n = n;
  h->precision = cfg->precision;
  h->cap = cfg->chi_cap;
  h->out_cap = cfg->out_cap;
  h->elem = 16;
  h->inst.resize(n);
  h->state.resize(n);
  h->infl_host.resize(n);
  std::vector<int> nslots(n);
  std::vector<double> props;
  for (int i = 0; i < n; ++i) {
    const otb_tempo_instance& s = ins[i];
    if (s.hs_dim < 1 || s.hs_dim > 3)
      return set_error(OTB_ERR_INVALID_ARG, "hs_dim must be 1..3 (Liouville dimension <= 9)");
    const int D = s.hs_dim * s.hs_dim;
    if (D > h->cap) return set_error(OTB_ERR_INVALID_ARG, "chi_cap must be >= D");
    if (D * h->cap > 1152) return set_error(OTB_ERR_INVALID_ARG, "chi_cap * D must be <= 1152");
    if (!(s.epsrel > 0.0) || !std::isfinite(s.epsrel))
      return set_error(OTB_ERR_INVALID_ARG, "epsrel must be positive and finite");
    if (!s.influences || !s.prop1 || !s.prop2 || !s.rho0)
      return set_error(OTB_ERR_INVALID_ARG, "null input array");
    const bool full = s.dkmax < 0;
    if (!full && s.n_influences < s.dkmax + 1)
      return set_error(OTB_ERR_INVALID_ARG, "need influences for dk = 0..dkmax");
    if (full && s.n_influences < 1)
      return set_error(OTB_ERR_INVALID_ARG, "need at least the dk=0 influence");
    h->Dmax = std::max(h->Dmax, D);
    InstDev& I = h->inst[i];
    I.D = D;
    I.dkmax = full ? (1 << 29) : s.dkmax;
    I.cap = h->cap;
    I.epsrel = s.epsrel;
    I.qr_delta = (float)cfg->qr_cut;
    I.out_cap = h->out_cap;
    I.out_origin = 0;
    const int want = full ? std::max(s.max_sites, 8) : s.dkmax + 2;
    nslots[i] = std::max(want, 2);
    const int ninfl = full ? s.n_influences : s.dkmax + 1;
    h->infl_host[i].assign(s.influences, s.influences + (size_t)ninfl * D * D * 2);
    I.prop_base = (long long)props.size() / 2;
    props.insert(props.end(), s.prop1, s.prop1 + 2 * D * D);
    props.insert(props.end(), s.prop2, s.prop2 + 2 * D * D);
    props.insert(props.end(), s.rho0, s.rho0 + 2 * D);
    I.ovr_base = (long long)props.size() / 2;
    props.insert(props.end(), (size_t)2 * D * D, 0.0);
    InstState& st = h->state[i];
    st.step = 0;
    st.nsites = 1;
    st.head = 0;
    st.status = 0;
    st.log_scale = 0.0;
    st.max_bond = 1;
    st.ovr_active = 0;
    st.splits = 0;
    st.sweeps64 = 0;
    st.sweeps32 = 0;
    st.flops_alg = 0.0;
    st.t_begin_ns = 0;
    st.t_end_ns = 0;
  }
  long long out_total = 0;
  for (int i = 0; i < n; ++i) {
    h->inst[i].out_base = out_total;
    out_total += (long long)h->out_cap * h->inst[i].D;
  }
  h->props_elems = (long long)props.size() / 2;
  if (!h->d_props.alloc(props.size() * sizeof(double))) return OTB_ERR_OOM;
  if (!check_cuda(cudaMemcpy(h->d_props.p, props.data(), props.size() * sizeof(double),
                             cudaMemcpyHostToDevice),
                  "upload props"))
    return OTB_ERR_CUDA;
  if (!h->d_out.alloc((size_t)out_total * 16)) return OTB_ERR_OOM;
  if (!check_cuda(cudaMemset(h->d_out.p, 0, (size_t)out_total * 16), "memset out")) return OTB_ERR_CUDA;
  if (!h->d_inst.alloc(sizeof(InstDev) * n)) return OTB_ERR_OOM;
  if (!h->d_state.alloc(sizeof(InstState) * n)) return OTB_ERR_OOM;
  if (!check_cuda(cudaMemcpy(h->d_state.p, h->state.data(), sizeof(InstState) * n,
                             cudaMemcpyHostToDevice),
                  "upload state"))
    return OTB_ERR_CUDA;
  otb_status st = layout_sites(h.get(), nslots, false);
  if (st) return st;
  st = upload_infl(h.get());
  if (st) return st;
  // initial site: rho0 as a (1, D, 1) tensor in slot 0; output step 0 = rho0
  for (int i = 0; i < n; ++i) {
    const InstDev& I = h->inst[i];
    const int D = I.D;
    std::vector<double> r0(ins[i].rho0, ins[i].rho0 + 2 * D);
    if (h->precision == OTB_PRECISION_MIXED) {
      // the mixed form's sites are double-float: each double x stored as the
      // float pair (hi, lo) with hi + lo = x to 48 bits
      std::vector<float> ffv(4 * D);
      for (int q = 0; q < 2 * D; ++q) {
        const float hi = (float)r0[q];
        ffv[2 * q] = hi;
        ffv[2 * q + 1] = (float)(r0[q] - (double)hi);
      }
      std::memcpy(r0.data(), ffv.data(), ffv.size() * sizeof(float));
    }
    if (!check_cuda(cudaMemcpy((char*)h->d_sites.p + I.site_base * h->elem, r0.data(),
                               r0.size() * sizeof(double), cudaMemcpyHostToDevice),
                    "init site"))
      return OTB_ERR_CUDA;
    int2 d0 = make_int2(1, 1);
    if (!check_cuda(cudaMemcpy((int2*)h->d_dims.p + I.dims_base, &d0, sizeof(int2),
                               cudaMemcpyHostToDevice),
                    "init dims"))
      return OTB_ERR_CUDA;
    // the output ring holds complex128 states in both forms
    if (!check_cuda(cudaMemcpy((double*)h->d_out.p + 2 * I.out_base, ins[i].rho0,
                               2 * D * sizeof(double), cudaMemcpyHostToDevice),
                    "init out"))
      return OTB_ERR_CUDA;
  }
  if ((st = upload_inst(h.get()))) return st;
  // processing order: most expensive first (memory length, then D)
  h->order.resize(n);
  std::iota(h->order.begin(), h->order.end(), 0);
  std::stable_sort(h->order.begin(), h->order.end(), [&](int a, int b) {
    const double ca = (double)std::min(h->inst[a].dkmax, 1 << 20) * h->inst[a].D * h->inst[a].D;
    const double cb = (double)std::min(h->inst[b].dkmax, 1 << 20) * h->inst[b].D * h->inst[b].D;
    return ca > cb;
  });
  if (!h->d_order.alloc(sizeof(int) * n) || !h->d_queue.alloc(sizeof(int))) return OTB_ERR_OOM;
  if (!check_cuda(cudaMemcpy(h->d_order.p, h->order.data(), sizeof(int) * n, cudaMemcpyHostToDevice),
                  "upload order"))
    return OTB_ERR_CUDA;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  // default launch shape: 3 CTAs of 256 threads per SM with 56 KiB smem;
  // CTAs of more than 256 threads (128 registers each) fill an SM alone
  const int per_sm = h->block > 256 ? 1 : 3;
  h->sms = std::max(sms, 1);
  h->grid = cfg->grid > 0 ? cfg->grid : std::max(1, std::min(n, per_sm * h->sms));
  // workspace for the widest default grid, so otb_tempo_set_launch can
  // switch shapes later (an explicit grid fixes it)
  h->grid_alloc = cfg->grid > 0 ? cfg->grid : std::max(h->grid, std::min(n, 3 * h->sms));
  if (h->smem_bytes == 0) h->smem_bytes = 56 * 1024;
  h->wcap = (long long)(h->cap * h->Dmax) * (h->cap * h->Dmax);
  h->work_stride = tempo_work_bytes(h->wcap);
  if (!h->d_work.alloc((size_t)h->grid_alloc * h->work_stride)) return OTB_ERR_OOM;
  *out = h.release();
  return OTB_OK;
}

extern "C" void otb_tempo_destroy(otb_tempo* h) { delete h; }

extern "C" otb_status otb_tempo_advance(otb_tempo* h, int32_t nsteps, void* stream) {
  if (!h || nsteps < 0) return set_error(OTB_ERR_INVALID_ARG, "bad arguments");
  if (nsteps == 0) return OTB_OK;
  // capacity checks that need host knowledge: site ring and influences
  for (int i = 0; i < h->n; ++i) {
    const InstDev& I = h->inst[i];
    if (I.dkmax >= (1 << 29)) {
      if (!check_cuda(cudaMemcpy(&h->state[i], (InstState*)h->d_state.p + i, sizeof(InstState),
                                 cudaMemcpyDeviceToHost),
                      "read state"))
        return OTB_ERR_CUDA;
      const int need_sites = h->state[i].nsites + nsteps + 1;
      if (need_sites > I.nslots)
        return set_error(OTB_ERR_INVALID_ARG, "full-memory run needs otb_tempo_reserve_sites first");
      if (h->state[i].step + nsteps > I.ninfl)
        return set_error(OTB_ERR_INVALID_ARG, "full-memory run needs influences up to dk = step");
    }
  }
  cudaStream_t s = (cudaStream_t)stream;
  if (!check_cuda(cudaMemsetAsync(h->d_queue.p, 0, sizeof(int), s), "reset queue")) return OTB_ERR_CUDA;
  // longest instance of the previous launch first (a launch waits on it)
  if (!check_cuda(launch_tempo_order((InstState*)h->d_state.p, (int*)h->d_order.p, h->n, s), "order"))
    return OTB_ERR_CUDA;
  TempoLaunch L;
  L.n = h->n;
  L.inst = (const InstDev*)h->d_inst.p;
  L.state = (InstState*)h->d_state.p;
  L.dims = (int2*)h->d_dims.p;
  L.sites = h->d_sites.p;
  L.infl = (const double*)h->d_infl.p;
  L.props = (const double*)h->d_props.p;
  L.out = (double*)h->d_out.p;
  L.work = h->d_work.p;
  L.work_stride = h->work_stride;
  L.wcap = h->wcap;
  L.queue = (int*)h->d_queue.p;
  L.order = (const int*)h->d_order.p;
  L.nsteps = nsteps;
  L.smem_bytes = 0;
  if (!check_cuda(launch_tempo(L, h->precision, h->grid, h->block, h->smem_bytes, s), "tempo launch"))
    return OTB_ERR_CUDA;
  return OTB_OK;
}

extern "C" otb_status otb_tempo_set_launch(otb_tempo* h, int32_t block, int32_t smem_kb, int32_t grid) {
  if (!h) return set_error(OTB_ERR_INVALID_ARG, "null handle");
  if (block != 0 && (block < 64 || block > 512 || block % 32 != 0))
    return set_error(OTB_ERR_INVALID_ARG, "block must be 0 or a multiple of 32 in [64, 512]");
  if (smem_kb < 0 || smem_kb > 200) return set_error(OTB_ERR_INVALID_ARG, "smem_kb must be in [0, 200]");
  if (grid < 0) return set_error(OTB_ERR_INVALID_ARG, "grid must be >= 0");
  h->block = block > 0 ? block : 256;
  h->smem_bytes = (smem_kb > 0 ? smem_kb : 56) * 1024;
  const int per_sm = h->block > 256 ? 1 : 3;
  const int want = grid > 0 ? grid : std::min(h->n, per_sm * h->sms);
  h->grid = std::max(1, std::min(want, h->grid_alloc));
  return OTB_OK;
}

extern "C" otb_status otb_tempo_get_info(otb_tempo* h, int32_t inst, otb_tempo_info* info) {
  otb_status st = check_inst(h, inst);
  if (st) return st;
  if (!info) return set_error(OTB_ERR_INVALID_ARG, "null info");
  if (!check_cuda(cudaMemcpy(&h->state[inst], (InstState*)h->d_state.p + inst, sizeof(InstState),
                             cudaMemcpyDeviceToHost),
                  "read state"))
    return OTB_ERR_CUDA;
  const InstState& s = h->state[inst];
  info->step = s.step;
  info->status = s.status;
  info->nsites = s.nsites;
  info->max_bond = s.max_bond;
  info->log_scale = s.log_scale;
  info->splits = s.splits;
  info->sweeps64 = s.sweeps64;
  info->sweeps32 = s.sweeps32;
  info->flops_alg = s.flops_alg;
  info->t_begin_ns = s.t_begin_ns;
  info->t_end_ns = s.t_end_ns;
  return OTB_OK;
}

extern "C" otb_status otb_tempo_read_states(otb_tempo* h, int32_t inst, int32_t first, int32_t count,
                                            double* out) {
  otb_status st = check_inst(h, inst);
  if (st) return st;
  if (!out || count < 0 || first < 0) return set_error(OTB_ERR_INVALID_ARG, "bad arguments");
  otb_tempo_info info;
  if ((st = otb_tempo_get_info(h, inst, &info))) return st;
  if (first + count - 1 > info.step) return set_error(OTB_ERR_INVALID_ARG, "step not computed yet");
  if (count > 0 && info.step - first >= h->out_cap)
    return set_error(OTB_ERR_INVALID_ARG, "step no longer held by the output ring");
  const InstDev& I = h->inst[inst];
  for (int k = 0; k < count; ++k) {
    const int s = first + k;
    const double* src = (const double*)h->d_out.p + 2 * (I.out_base + (long long)(s % h->out_cap) * I.D);
    if (!check_cuda(cudaMemcpy(out + (size_t)2 * I.D * k, src, sizeof(double) * 2 * I.D,
                               cudaMemcpyDeviceToHost),
                    "read states"))
      return OTB_ERR_CUDA;
  }
  return OTB_OK;
}

extern "C" otb_status otb_tempo_read_all_states(otb_tempo* h, int32_t first, int32_t count,
                                                double* out) {
  if (!h || !out) return set_error(OTB_ERR_INVALID_ARG, "bad arguments");
  // fast path: whole ring in one copy when the ring covers [0, out_cap) and
  // the request is exactly that window with uniform D
  std::vector<double> ring((size_t)2 * (h->inst.back().out_base + (long long)h->out_cap * h->inst.back().D));
  if (!check_cuda(cudaMemcpy(ring.data(), h->d_out.p, ring.size() * sizeof(double), cudaMemcpyDeviceToHost),
                  "read ring"))
    return OTB_ERR_CUDA;
  if (!check_cuda(cudaMemcpy(h->state.data(), h->d_state.p, sizeof(InstState) * h->n, cudaMemcpyDeviceToHost),
                  "read state"))
    return OTB_ERR_CUDA;
  size_t off = 0;
  for (int i = 0; i < h->n; ++i) {
    if (h->state[i].status != 0)
      return set_error(h->state[i].status, "instance " + std::to_string(i) + " stopped at step " +
                                               std::to_string(h->state[i].step) + " with status " +
                                               std::to_string(h->state[i].status));
  }
  for (int i = 0; i < h->n; ++i) {
    const InstDev& I = h->inst[i];
    const int step = h->state[i].step;
    for (int k = 0; k < count; ++k) {
      const int s = first + k;
      if (s > step || step - s >= h->out_cap)
        return set_error(OTB_ERR_INVALID_ARG, "step outside the output ring");
      const double* src = ring.data() + 2 * (I.out_base + (long long)(s % h->out_cap) * I.D);
      std::memcpy(out + off, src, sizeof(double) * 2 * I.D);
      off += 2 * I.D;
    }
  }
  return OTB_OK;
}

extern "C" otb_status otb_tempo_bond_dims(otb_tempo* h, int32_t inst, int32_t* out, int32_t cap,
                                          int32_t* count) {
  otb_status st = check_inst(h, inst);
  if (st) return st;
  otb_tempo_info info;
  if ((st = otb_tempo_get_info(h, inst, &info))) return st;
  const InstDev& I = h->inst[inst];
  const InstState& s = h->state[inst];
  std::vector<int2> dims(I.nslots);
  if (!check_cuda(cudaMemcpy(dims.data(), (int2*)h->d_dims.p + I.dims_base, sizeof(int2) * I.nslots,
                             cudaMemcpyDeviceToHost),
                  "read dims"))
    return OTB_ERR_CUDA;
  const int nb = std::max(0, s.nsites - 1);
  if (count) *count = nb;
  for (int k = 0; k < nb && k < cap; ++k) out[k] = dims[(s.head + k) % I.nslots].y;
  return OTB_OK;
}

extern "C" otb_status otb_tempo_set_influence(otb_tempo* h, int32_t inst, int32_t dk, const double* mat) {
  otb_status st = check_inst(h, inst);
  if (st) return st;
  if (!mat || dk < 0) return set_error(OTB_ERR_INVALID_ARG, "bad arguments");
  const int D = h->inst[inst].D;
  std::vector<double>& v = h->infl_host[inst];
  const size_t need = (size_t)(dk + 1) * D * D * 2;
  if (v.size() < need) v.resize(need, 0.0);
  std::memcpy(v.data() + (size_t)dk * D * D * 2, mat, sizeof(double) * D * D * 2);
  if ((st = upload_infl(h))) return st;
  return upload_inst(h);
}

extern "C" otb_status otb_tempo_set_propagators(otb_tempo* h, int32_t inst, const double* p1,
                                                const double* p2) {
  otb_status st = check_inst(h, inst);
  if (st) return st;
  if (!p1 || !p2) return set_error(OTB_ERR_INVALID_ARG, "null propagator");
  const InstDev& I = h->inst[inst];
  const size_t b = (size_t)I.D * I.D * 2 * sizeof(double);
  double* base = (double*)h->d_props.p + 2 * I.prop_base;
  if (!check_cuda(cudaMemcpy(base, p1, b, cudaMemcpyHostToDevice), "set prop1")) return OTB_ERR_CUDA;
  if (!check_cuda(cudaMemcpy(base + 2 * I.D * I.D, p2, b, cudaMemcpyHostToDevice), "set prop2"))
    return OTB_ERR_CUDA;
  return OTB_OK;
}

extern "C" otb_status otb_tempo_set_all_propagators(otb_tempo* h, const double* p1, const double* p2,
                                                    void* stream) {
  if (!h) return set_error(OTB_ERR_INVALID_ARG, "null handle");
  if (!p1 || !p2) return set_error(OTB_ERR_INVALID_ARG, "null propagator");
  cudaStream_t s = (cudaStream_t)stream;
  const int n = (int)h->inst.size();
  bool uniform = true;
  for (int i = 1; i < n && uniform; ++i)
    uniform = h->inst[i].D == h->inst[0].D &&
              h->inst[i].prop_base - h->inst[i - 1].prop_base ==
                  (n > 1 ? h->inst[1].prop_base - h->inst[0].prop_base : 0);
  if (uniform && n > 1) {
    // one strided copy per propagator: instance i's P1 / P2 sit at a fixed pitch
    const int D = h->inst[0].D;
    const size_t w = (size_t)D * D * 2 * sizeof(double);
    const size_t pitch = (size_t)(h->inst[1].prop_base - h->inst[0].prop_base) * 2 * sizeof(double);
    double* base = (double*)h->d_props.p + 2 * h->inst[0].prop_base;
    if (!check_cuda(cudaMemcpy2DAsync(base, pitch, p1, w, w, n, cudaMemcpyHostToDevice, s), "set all prop1") ||
        !check_cuda(cudaMemcpy2DAsync(base + 2 * D * D, pitch, p2, w, w, n, cudaMemcpyHostToDevice, s),
                    "set all prop2"))
      return OTB_ERR_CUDA;
    return OTB_OK;
  }
  size_t off = 0;
  for (int i = 0; i < n; ++i) {
    const InstDev& I = h->inst[i];
    const size_t b = (size_t)I.D * I.D * 2 * sizeof(double);
    double* base = (double*)h->d_props.p + 2 * I.prop_base;
    if (!check_cuda(cudaMemcpyAsync(base, p1 + off, b, cudaMemcpyHostToDevice, s), "set prop1") ||
        !check_cuda(cudaMemcpyAsync(base + 2 * I.D * I.D, p2 + off, b, cudaMemcpyHostToDevice, s), "set prop2"))
      return OTB_ERR_CUDA;
    off += (size_t)I.D * I.D * 2;
  }
  return OTB_OK;
}

extern "C" otb_status otb_tempo_set_first_influence(otb_tempo* h, int32_t inst, const double* mat) {
  otb_status st = check_inst(h, inst);
  if (st) return st;
  const InstDev& I = h->inst[inst];
  if (!check_cuda(cudaMemcpy(&h->state[inst], (InstState*)h->d_state.p + inst, sizeof(InstState),
                             cudaMemcpyDeviceToHost),
                  "read state"))
    return OTB_ERR_CUDA;
  if (mat) {
    if (!check_cuda(cudaMemcpy((double*)h->d_props.p + 2 * I.ovr_base, mat,
                               sizeof(double) * 2 * I.D * I.D, cudaMemcpyHostToDevice),
                    "set override"))
      return OTB_ERR_CUDA;
  }
  h->state[inst].ovr_active = mat ? 1 : 0;
  if (!check_cuda(cudaMemcpy((InstState*)h->d_state.p + inst, &h->state[inst], sizeof(InstState),
                             cudaMemcpyHostToDevice),
                  "write state"))
    return OTB_ERR_CUDA;
  return OTB_OK;
}

extern "C" otb_status otb_tempo_reserve_sites(otb_tempo* h, int32_t nslots) {
  if (!h || nslots < 2) return set_error(OTB_ERR_INVALID_ARG, "bad arguments");
  std::vector<int> ns(h->n);
  bool grow = false;
  for (int i = 0; i < h->n; ++i) {
    ns[i] = std::max(h->inst[i].nslots, (int)nslots);
    grow = grow || ns[i] != h->inst[i].nslots;
  }
  if (!grow) return OTB_OK;
  otb_status st = layout_sites(h, ns, true);
  if (st) return st;
  return upload_inst(h);
}
