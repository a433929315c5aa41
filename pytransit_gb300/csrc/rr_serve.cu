// Per-request set-up of the serving layer in one call: the host-to-device
// copy of the request's staged inputs, the FP32-pair time split, the fused
// split prologue (RoadRunner: rr_prepare_split_ld; transmission spectroscopy:
// rr_ts_prepare_split_ld), the request's descriptor for the persistent flux
// kernel, its stated error bound and the bound's copy to a pinned host slot,
// all enqueued on one stream.  A Python host issuing these one by one spends
// more time in argument conversion than the GPU spends on a small request.
#include "rr_internal.h"

using namespace rr;

extern "C" {

int rr_serve_setup(int kind, const rr_serve_setup_args* a, void* stream) {
  if (!a || (kind != 0 && kind != 1) || a->npt < 0 || a->npv < 1 || a->npb < 1 || a->nlc < 1 || a->ng < 2)
    return RR_ERR_ARG;
  cudaStream_t s = as_stream(stream);
  const int npt = (int)a->npt, npv = (int)a->npv, npb = (int)a->npb, nlc = (int)a->nlc, ng = (int)a->ng;
  const int nep = (int)a->nep, npar = (int)a->npar, nz = (int)a->nz;
  if (a->n_in > 0) {
    const cudaError_t e = cudaMemcpyAsync(a->dst, a->stage, (size_t)a->n_in, cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) {
      set_cuda_error(e, "rr_serve_setup: inputs");
      return RR_ERR_CUDA;
    }
  }
  int st = rr_time_split(a->time, a->lcids, npt, a->t_ref, a->times_ff, stream);
  if (st) return st;
  rr_serve_request* d = a->desc;
  if (kind == 0) {
    st = rr_prepare_split_ld(a->t_ref, a->t_abs, a->k, (int)a->nkc, a->t0, nep, nep, a->p, a->a, a->inc, a->e, a->w,
                             npv, nlc, npb, a->pbids, a->epids, a->nsamples, a->exptimes, (int)a->law, a->ldc, npar,
                             a->mu, nz, a->basis, (int)a->nb, a->weights, (int)a->nk, ng, a->dk, a->kmin, a->kmax,
                             a->z_edges, a->ldp, a->istar, a->ws, (size_t)a->wsb, stream);
    if (st) return st;
    if (d) {
      const float *orb, *lc, *ldm;
      rr_full_split_tables(a->ws, npv, npb, nlc, nep, ng, &orb, &lc, &ldm);
      d->times_ff = a->times_ff;
      d->lcids = a->lcids;
      d->orb32 = orb; d->lc32 = lc; d->ldm = ldm;
      d->flux = a->flux; d->ldflux = a->ldflux;
      d->npt = npt; d->npv = npv; d->nlc = nlc; d->npb = npb; d->ng = ng; d->kind = 0;
      d->inv_dg = (float)(1.0 / a->dg); d->exptime0 = 0.0f; d->dg = a->dg;
      d->nsamples0 = 0; d->pad = 0;
    }
    st = rr_split_error_bounds(a->p, a->a, a->inc, a->e, a->w, npv, npb, nlc, nep, ng, a->dg, a->ws, a->bnd,
                               a->bmax, stream);
  } else {
    st = rr_ts_prepare_split_ld((int)a->law, a->ldc, npar, a->mu, a->t_ref, a->t_abs, a->k, a->t0, a->p, a->a,
                                a->inc, a->e, a->w, npv, npb, a->exptime0, ng, nz, a->z_edges, a->ws,
                                (size_t)a->wsb, stream);
    if (st) return st;
    if (d) {
      const void *orb, *ch, *ldm;
      rr_ts_tables(a->ws, 1, npv, npb, ng, &orb, &ch, &ldm);
      d->times_ff = a->times_ff;
      d->lcids = nullptr;
      d->orb32 = static_cast<const float*>(orb); d->lc32 = static_cast<const float*>(ch);
      d->ldm = static_cast<const float*>(ldm);
      d->flux = a->flux; d->ldflux = a->ldflux;
      d->npt = npt; d->npv = npv; d->nlc = 1; d->npb = npb; d->ng = ng; d->kind = 1;
      d->inv_dg = (float)(1.0 / a->dg); d->exptime0 = (float)a->exptime0; d->dg = a->dg;
      d->nsamples0 = (int)a->nsamples0; d->pad = 0;
    }
    st = rr_ts_split_error_bounds(a->p, a->a, a->inc, a->e, a->w, npv, npb, ng, a->dg, (int)a->nsamples0,
                                  a->exptime0, a->ws, a->bnd, a->bmax, stream);
  }
  if (st) return st;
  if (a->bound_host) {
    const cudaError_t e = cudaMemcpyAsync(a->bound_host, a->bmax, sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess) {
      set_cuda_error(e, "rr_serve_setup: bound");
      return RR_ERR_CUDA;
    }
  }
  return RR_OK;
}

void rr_serve_setup_args_size(int* size) { *size = (int)sizeof(rr_serve_setup_args); }

}  // extern "C"
