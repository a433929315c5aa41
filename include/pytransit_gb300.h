/*
 * pytransit_gb300 — C ABI of the GB300-native RoadRunner transit-model path.
 *
 * Every entry point takes device pointers (allocated by the caller), plain
 * sizes and a CUDA stream (as void*; NULL = legacy default stream), launches
 * asynchronously on that stream and returns an int status (RR_OK = 0).  The
 * library never allocates device memory: per-call scratch is a caller-owned
 * workspace sized by the matching *_workspace_bytes() function.
 *
 * Array layouts are row-major, as the reference's numpy arrays:
 *   times[npt] f64, k[npv, nkc] (nkc = 1 or npb), t0[npv, ldt0] (column =
 *   epoch id), p/a/inc/e/w[npv] f64, lcids[npt] int32, pbids/epids/nsamples
 *   [nlc] int32, exptimes[nlc] f64, ldp[npv, npb, nz], istar[npv, npb],
 *   weights[nk, ng, nz], flux[npv, ldflux] (ldflux >= npt).
 *
 * Reference: hpparvi/PyTransit 2.8.1 (paths below are inside that project).
 */
#ifndef PYTRANSIT_GB300_H
#define PYTRANSIT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
#define RR_OK 0
#define RR_ERR_SHAPE 1     /* k is neither [npv,1] nor [npv,npb] (model_full.py:18-19) */
#define RR_ERR_ARG 2       /* a size or pointer argument is invalid */
#define RR_ERR_WORKSPACE 3 /* workspace smaller than *_workspace_bytes() */
#define RR_ERR_CUDA 4      /* a CUDA launch failed; see rr_last_cuda_error() */
#define RR_ERR_LAW 5       /* unknown limb-darkening law id */
#define RR_ERR_TIMEOUT 6   /* a bounded device wait ran out */

/* Limb-darkening law ids: the named laws of RoadRunnerModel.ldmodels
 * (pytransit/models/roadrunner/rrmodel.py:48-58). */
#define RR_LD_UNIFORM 0
#define RR_LD_LINEAR 1
#define RR_LD_QUADRATIC 2
#define RR_LD_QUADRATIC_TRI 3
#define RR_LD_NONLINEAR 4
#define RR_LD_GENERAL 5
#define RR_LD_SQUARE_ROOT 6
#define RR_LD_LOGARITHMIC 7
#define RR_LD_EXPONENTIAL 8
#define RR_LD_POWER_2 9
#define RR_LD_POWER_2_PM 10

int rr_abi_version(void);
const char *rr_status_string(int status);
/* The last error an entry point recorded on this host thread: where it
 * happened and the CUDA error's text, or the library's own message for some
 * argument errors; "no error" before the first. */
const char *rr_last_cuda_error(void);

/* ---- model initialisation ------------------------------------------------ */

/* Replaces calculate_weights_3d (pytransit/models/roadrunner/common.py:189-223).
 * Fills W64[nk, ng, nz] (and W32, an FP32 copy, when non-NULL) from the
 * radial grid ze[nz] (device).  Writes dk = (kmax-kmin)/nk and dg to the host
 * pointers (the reference's definitions, including dk's 1/nk). */
int rr_weights_3d(int nk, double kmin, double kmax, const double *ze, int nz, int ng,
                  double *W64, float *W32, double *dk, double *dg, void *stream);

/* ---- data (set_data) ----------------------------------------------------- */

/* Part of TransitModel.set_data (pytransit/models/transitmodel.py:56-125) for
 * the split-precision path.  times_ff holds rr_time_split_floats(npt) floats:
 * first the FP32 pairs times_ff[2*i] = hi, [2*i+1] = lo with
 * hi + lo = times[i] - t_ref to ~2^-48 relative, then (at float offset
 * 2 * round_up(npt, 2)) one float4 per 128-point tile: the tile's smallest and
 * largest hi and its light-curve id (int bits), or -1 when the tile spans
 * several light curves. */
size_t rr_time_split_floats(int npt);
int rr_time_split(const double *times, const int32_t *lcids, int npt, double t_ref, float *times_ff,
                  void *stream);

/* ---- limb-darkening layer -------------------------------------------------- */

/* Replaces evaluate_ld / evaluate_ldi (pytransit/models/numba/ldmodels.py:143-174)
 * and the numerical disk integral of rrmodel.py:219-227 (laws without ldi_*):
 * ldc[npv, npb, npar] -> ldp[npv, npb, nz] at mu[nz], istar[npv, npb]. */
int rr_ld_tables_f64(int law, const double *ldc, int npv, int npb, int npar, const double *mu,
                     int nz, double *ldp, double *istar, void *stream);
/* Same in FP32 (the split-precision path's LD layer). */
int rr_ld_tables_f32(int law, const double *ldc, int npv, int npb, int npar, const double *mu,
                     int nz, float *ldp, float *istar, void *stream);

/* ---- full RoadRunner model --------------------------------------------------- */

/* Workspace for rr_full_f64 / rr_full_split. */
size_t rr_full_f64_workspace_bytes(int npv, int npb, int ng);
size_t rr_full_split_workspace_bytes(int npv, int npb, int nlc, int nep, int ng);

/* Replaces rr_full (pytransit/models/roadrunner/model_full.py:9-100) and
 * rr_simple (model_simple.py:12-80), all in FP64: per-pv prologue (validity,
 * LD means, orbit, bounding box) then flux[npv, npt].  Invalid parameter
 * vectors (a NaN or <= 1, e < 0, ldp[pv,0,0] NaN) give NaN rows. */
int rr_full_f64(const double *times, int npt, const double *k, int nkc, const double *t0, int ldt0,
                const double *p, const double *a, const double *inc, const double *e,
                const double *w, int npv, int nlc, int npb, const int32_t *lcids,
                const int32_t *pbids, const int32_t *epids, const int32_t *nsamples,
                const double *exptimes, const double *ldp, const double *istar,
                const double *weights, int nk, int ng, int nz, double dk, double kmin,
                double kmax, double dg, const double *z_edges, void *workspace,
                size_t workspace_bytes, double *flux, int ldflux, void *stream);

/* Same model, split precision: FP64 orbit (Taylor coefficients, contact
 * points) and phase reduction data per parameter vector; per point an FP32
 * pair phase reduction (times_ff from rr_time_split with the same t_ref,
 * t_absmax = max |times - t_ref|), FP32 z, interpolation and flux deficit,
 * supersamples spread over warp lanes and summed with shuffles.  ldp/istar
 * from rr_ld_tables_f32, weights = the FP32 table.  flux is FP32. */
int rr_full_split(const float *times_ff, double t_ref, double t_absmax, int npt, const double *k,
                  int nkc, const double *t0, int ldt0, int nep, const double *p, const double *a,
                  const double *inc, const double *e, const double *w, int npv, int nlc, int npb,
                  const int32_t *lcids, const int32_t *pbids, const int32_t *epids,
                  const int32_t *nsamples, const double *exptimes, const float *ldp,
                  const float *istar, const float *weights, int nk, int ng, int nz, double dk,
                  double kmin, double kmax, double dg, const double *z_edges, void *workspace,
                  size_t workspace_bytes, float *flux, int ldflux, void *stream);

/* Affine LD laws (all named laws except power-2 and power-2-pm) are
 * I(mu) = sum_b coef_b phi_b(mu); their LD means need only the per-k-row
 * basis tables B[nk, nb, ng] = W @ phi_b (nb = rr_basis_count(law, npar), 0
 * for the other laws), built once per model by rr_basis_tables (B32 may be
 * NULL).  Passing them to rr_prepare_* (law, ldc[npv, npb, npar], basis, nb)
 * replaces the per-pv W @ ldp products of model_full.py:46-51; basis = NULL
 * selects the generic products. */
int rr_basis_count(int law, int npar);
int rr_basis_tables(int law, int npar, const double *mu, int nz, const double *W64, int nk, int ng,
                    double *B64, float *B32, void *stream);

/* The two stages of rr_full_f64, callable separately (the workspace carries
 * the per-parameter-vector tables from one to the other): the prologue of
 * model_full.py:39-71 and the flux loop of model_full.py:75-99. */
int rr_prepare_f64(const double *k, int nkc, const double *p, const double *a, const double *inc,
                   const double *e, const double *w, int npv, int npb, const double *ldp,
                   const double *weights, int nk, int ng, int nz, double dk, double kmin, double kmax,
                   const double *z_edges, void *workspace, size_t workspace_bytes, void *stream,
                   int law, const double *ldc, int npar, const double *basis, int nb);
int rr_flux_f64(const double *times, int npt, const double *k, int nkc, const double *t0, int ldt0,
                const double *p, int npv, int nlc, int npb, const int32_t *lcids, const int32_t *pbids,
                const int32_t *epids, const int32_t *nsamples, const double *exptimes,
                const double *istar, int ng, double dg, const void *workspace, double *flux, int ldflux,
                void *stream);

/* FP64 summaries of the 128-point time tiles, for rr_flux_f64_culled_range:
 * tiles64[4 * tile + 0..3] = (earliest time, latest time, light curve or -1
 * when the tile holds several, 0); rr_time_tiles_f64_doubles(npt) doubles.
 * Made once per data set, as rr_time_split (transitmodel.py:56-125). */
size_t rr_time_tiles_f64_doubles(int npt);
int rr_time_tiles_f64(const double *times, const int32_t *lcids, int npt, double *tiles64, void *stream);

/* rr_flux_f64_range with the fold (model_full.py:88-91) done once per tile
 * for the tiles that reach no box.  The reference's epoch and tc are
 * non-decreasing in t with its own rounding, so a one-light-curve tile with
 * the same epoch at both ends, whose two ends' tc miss the box, holds 1.0 at
 * every point: the same bits as rr_flux_f64, for a fraction of its FP64
 * work.  The other tiles take the per-point arithmetic of rr_flux_f64. */
int rr_flux_f64_culled_range(const double *times, const double *tiles64, int npt, const double *k, int nkc,
                             const double *t0, int ldt0, const double *p, int npv, int nlc, int npb,
                             const int32_t *lcids, const int32_t *pbids, const int32_t *epids,
                             const int32_t *nsamples, const double *exptimes, const double *istar, int ng,
                             double dg, const void *workspace, int pv0, int pv1, double *flux, int ldflux,
                             void *stream);

/* rr_flux_f64 for the parameter vectors [pv0, pv1) of the prepared
 * workspace, into their own rows flux[pv1 - pv0, ldflux] (the arrays k, t0,
 * p, istar are the whole population's).  Lets a caller copy the flux of one
 * range to the host while the next is computed. */
int rr_flux_f64_range(const double *times, int npt, const double *k, int nkc, const double *t0, int ldt0,
                      const double *p, int npv, int nlc, int npb, const int32_t *lcids, const int32_t *pbids,
                      const int32_t *epids, const int32_t *nsamples, const double *exptimes,
                      const double *istar, int ng, double dg, const void *workspace, int pv0, int pv1,
                      double *flux, int ldflux, void *stream);

/* The two stages of rr_full_split: the prologue writes the per-parameter-vector
 * and per-(pv, light curve) tables into the workspace, the flux stage reads
 * only those tables, the FP32-pair times and the light-curve ids. */
int rr_prepare_split(double t_ref, double t_absmax, const double *k, int nkc, const double *t0, int ldt0,
                     int nep, const double *p, const double *a, const double *inc, const double *e,
                     const double *w, int npv, int nlc, int npb, const int32_t *pbids,
                     const int32_t *epids, const int32_t *nsamples, const double *exptimes,
                     const float *ldp, const float *istar, const float *weights, int nk, int ng, int nz,
                     double dk, double kmin, double kmax, const double *z_edges, void *workspace,
                     size_t workspace_bytes, void *stream, int law, const double *ldc, int npar,
                     const float *basis, int nb);
int rr_flux_split(const float *times_ff, int npt, const int32_t *lcids, int npv, int nlc, int npb, int ng,
                  double dg, const void *workspace, float *flux, int ldflux, void *stream);
/* rr_ld_tables_f32 followed by rr_prepare_split, as one launch for the
 * affine laws with an analytic disk integral (uniform, linear, quadratic,
 * quadratic-tri) given their basis tables: ldp[npv, npb, nz] and
 * istar[npv, npb] are written as rr_ld_tables_f32 writes them, and the
 * workspace is filled as rr_prepare_split fills it (the LD profile of
 * rrmodel.py:212-227 and the prologue of model_full.py:39-71).  For other
 * laws, no basis, or npb * (npar + 1) > 128, the two stages run one after
 * the other with the same arguments. */
int rr_prepare_split_ld(double t_ref, double t_absmax, const double *k, int nkc, const double *t0, int ldt0,
                        int nep, const double *p, const double *a, const double *inc, const double *e,
                        const double *w, int npv, int nlc, int npb, const int32_t *pbids,
                        const int32_t *epids, const int32_t *nsamples, const double *exptimes, int law,
                        const double *ldc, int npar, const double *mu, int nz, const float *basis, int nb,
                        const float *weights, int nk, int ng, double dk, double kmin, double kmax,
                        const double *z_edges, float *ldp, float *istar, void *workspace,
                        size_t workspace_bytes, void *stream);
/* rr_flux_split for the parameter vectors [pv0, pv1) of a workspace prepared
 * for npv: flux[pv1 - pv0, ldflux] holds those rows.  Lets a caller compute
 * the flux in pv chunks and move each chunk to the host while the next one
 * is computed. */
int rr_flux_split_range(const float *times_ff, int npt, const int32_t *lcids, int npv, int nlc, int npb, int ng,
                        double dg, const void *workspace, int pv0, int pv1, float *flux, int ldflux,
                        void *stream);

/* rr_flux_split_range that stores only what can differ from 1: the 128-point
 * tiles whose times reach a transit window (every point of such a tile) and
 * the NaN rows of invalid parameter vectors.  Every other point of
 * flux[pv1 - pv0, ldflux] must already hold 1.0, the value the reference
 * gives every point outside the bounding box (model_full.py:90-91).  flux
 * may be device memory or page-locked host
 * memory (cudaHostAlloc / cudaHostRegister), which the kernel writes through
 * its device address; pageable host memory is rejected (RR_ERR_ARG).  With
 * rr_host_fill_f32 this moves one bit per culled tile instead of its 512
 * bytes: the host sets a chunk of rows to 1 while the GPU writes the transit
 * tiles of the chunk before it. */
int rr_flux_split_transits(const float *times_ff, int npt, const int32_t *lcids, int npv, int nlc, int npb,
                           int ng, double dg, const void *workspace, int pv0, int pv1, float *flux, int ldflux,
                           void *stream);

/* Host memory fill on the library's own threads: dst[0..n) = value, split
 * over nthreads threads (the calling thread included; nthreads <= 0 or 1:
 * the calling thread alone).  The threads are started on first use and kept;
 * a process forked after that starts its own.  No GPU work.  Returns 0, or
 * RR_ERR_ARG for dst NULL with n > 0. */
int rr_host_fill_f32(float *dst, size_t n, float value, int nthreads);
int rr_host_fill_f64(double *dst, size_t n, double value, int nthreads);

/* rr_flux_split_range and rr_flux_split_transits with FP64 output rows (the
 * reference's output type, model_full.py:75): each FP32 result widened
 * exactly, the same values as the FP32 rows. */
int rr_flux_split_range_f64(const float *times_ff, int npt, const int32_t *lcids, int npv, int nlc, int npb,
                            int ng, double dg, const void *workspace, int pv0, int pv1, double *flux, int ldflux,
                            void *stream);
int rr_flux_split_transits_f64(const float *times_ff, int npt, const int32_t *lcids, int npv, int nlc, int npb,
                               int ng, double dg, const void *workspace, int pv0, int pv1, double *flux,
                               int ldflux, void *stream);

/* ---- transmission-spectroscopy model --------------------------------------- */

/* Replaces tsmodel_serial (pytransit/models/roadrunner/model_trspec.py:12-93)
 * behind TransmissionSpectroscopyModel.evaluate (tsmodel.py:46-130): k[npv, npb]
 * one radius ratio per channel, t0[npv], ldp[npv, npb, nz], istar[npv, npb];
 * weights = NULL uses the 2D table at the mean radius ratio (the reference's
 * default), a 3D table the reference's precompute_weights rule.  Only
 * nsamples0 and exptime0 (the first light curve's) are used, as in the
 * reference.  -> flux[npv, npb, ldflux]. */
size_t rr_ts_workspace_bytes(int split, int npv, int npb, int ng);
int rr_ts_f64(const double *times, int npt, const double *k, const double *t0, const double *p,
              const double *a, const double *inc, const double *e, const double *w, int npv, int npb,
              int nsamples0, double exptime0, const double *ldp, const double *istar, const double *weights,
              int nk, int ng, int nz, double dk, double kmin, double kmax, double dg, const double *z_edges,
              void *workspace, size_t workspace_bytes, double *flux, int ldflux, void *stream);
/* The two halves of rr_ts_split (for callers that keep the per-pv tables
 * between calls, such as the serving loop): rr_ts_prepare_split writes the
 * per-pv records, the channel records and the LD means into the workspace
 * (tsmodel_serial's per-pv prologue, model_trspec.py:36-66); rr_ts_flux_split
 * evaluates the light curves from them (model_trspec.py:72-93).
 * rr_ts_tables gives the addresses of those tables inside the workspace. */
int rr_ts_prepare_split(double t_ref, double t_absmax, const double *k, const double *t0, const double *p,
                        const double *a, const double *inc, const double *e, const double *w, int npv, int npb,
                        double exptime0, const float *ldp, const float *istar, const float *weights, int nk, int ng,
                        int nz, double dk, double kmin, double kmax, const double *z_edges, void *workspace,
                        size_t workspace_bytes, void *stream);
int rr_ts_flux_split(const float *times_ff, int npt, int npv, int npb, int nsamples0, double exptime0, int ng,
                     double dg, const void *workspace, float *flux, int ldflux, void *stream);
/* rr_ts_flux_split for the parameter vectors [pv0, pv1) of a workspace
 * prepared for npv: flux holds their rows only, flux[pv1 - pv0, npb, ldflux]. */
int rr_ts_flux_split_range(const float *times_ff, int npt, int npv, int npb, int nsamples0, double exptime0, int ng,
                           double dg, const void *workspace, int pv0, int pv1, float *flux, int ldflux, void *stream);
void rr_ts_tables(void *workspace, int split, int npv, int npb, int ng, const void **orb, const void **ch,
                  const void **ldm);
/* The prologue for a named law with the default 2D table (TSModel.evaluate
 * with a string ldmodel, tsmodel.py:46-130: evaluate_ld / evaluate_ldi or the
 * 200-point trapezoid, then tsmodel_serial's per-pv prologue,
 * model_trspec.py:36-66), one launch: ldc[npv, npb, npar] on the mu grid
 * mu[nz] instead of ldp / istar.  rr_ts_flux_f64 is the plain path's flux
 * half (model_trspec.py:72-93). */
int rr_ts_prepare_split_ld(int law, const double *ldc, int npar, const double *mu, double t_ref, double t_absmax,
                           const double *k, const double *t0, const double *p, const double *a, const double *inc,
                           const double *e, const double *w, int npv, int npb, double exptime0, int ng, int nz,
                           const double *z_edges, void *workspace, size_t workspace_bytes, void *stream);
int rr_ts_prepare_f64_ld(int law, const double *ldc, int npar, const double *mu, const double *k, const double *t0,
                         const double *p, const double *a, const double *inc, const double *e, const double *w,
                         int npv, int npb, double exptime0, int ng, int nz, const double *z_edges, void *workspace,
                         size_t workspace_bytes, void *stream);
int rr_ts_flux_f64(const double *times, int npt, const double *t0, const double *p, int npv, int npb, int nsamples0,
                   double exptime0, int ng, double dg, const void *workspace, double *flux, int ldflux,
                   void *stream);
/* rr_ts_flux_f64 with the fold (model_trspec.py:74-76) once per 128-point
 * tile for the tiles that reach no box, from the FP64 tile summaries of
 * rr_time_tiles_f64: the fold is non-decreasing in t with the reference's
 * rounding, so such a tile is 1.0 at every point; the same bits as
 * rr_ts_flux_f64. */
int rr_ts_flux_f64_culled(const double *times, const double *tiles64, int npt, const double *t0, const double *p,
                          int npv, int npb, int nsamples0, double exptime0, int ng, double dg, const void *workspace,
                          double *flux, int ldflux, void *stream);
/* Same, split precision (times_ff and t_ref/t_absmax as rr_full_split). */
int rr_ts_split(const float *times_ff, double t_ref, double t_absmax, int npt, const double *k,
                const double *t0, const double *p, const double *a, const double *inc, const double *e,
                const double *w, int npv, int npb, int nsamples0, double exptime0, const float *ldp,
                const float *istar, const float *weights, int nk, int ng, int nz, double dk, double kmin,
                double kmax, double dg, const double *z_edges, void *workspace, size_t workspace_bytes,
                float *flux, int ldflux, void *stream);

/* ---- Gaussian log-likelihood and its gradient ----------------------------- */

/* Fused model + Gaussian log-likelihood per parameter vector
 * (pytransit/lpf/loglikelihood/wnloglikelihood.py:23-35, lpf.py:51-66):
 *   lnl[pv] = sum_i -log(sigma_lc(i)) - log(2 pi)/2 - ((obs_i - flux[pv, i]) / sigma_lc(i))^2 / 2
 * with sigma[nlc] one noise level per light curve; the flux is never stored.
 * With grad != NULL also d lnl / d theta, grad[npv, ngrad] with columns
 * [k (nkc)][t0 (nep)][p, a, i, e, w][ldc (npb x npar)], ngrad =
 * rr_lnlike_ngrad(); the gradient is that of the discretised model (table
 * interpolations, kite area, orbit Taylor coefficients), recomputing z per
 * sample.  The reference has no adjoint (its dfdk/dfdb, common.py:105-128, are
 * unused partials).  Named LD laws only (law, ldc[npv, npb, npar], npar <= 4);
 * ldp/istar as from rr_ld_tables_*. */
int rr_lnlike_ngrad(int nkc, int nep, int npb, int npar);
size_t rr_lnlike_workspace_bytes(int split, int npv, int npb, int nlc, int nep, int ng, int npar, int npt,
                                 int nkc);
int rr_lnlike_f64(int law, const double *ldc, int npar, const double *mu, const double *times, int npt,
                  const double *k, int nkc, const double *t0, int ldt0, int nep, const double *p,
                  const double *a, const double *inc, const double *e, const double *w, int npv, int nlc,
                  int npb, const int32_t *lcids, const int32_t *pbids, const int32_t *epids,
                  const int32_t *nsamples, const double *exptimes, const double *ldp, const double *istar,
                  const double *weights, int nk, int ng, int nz, double dk, double kmin, double kmax,
                  double dg, const double *z_edges, const double *obs, const double *sigma, void *workspace,
                  size_t workspace_bytes, double *lnl, double *grad, void *stream);
/* Same, split precision (FP32 per-sample arithmetic and residuals formed from
 * the deficit, FP64 block sums). */
int rr_lnlike_split(int law, const double *ldc, int npar, const double *mu, const float *times_ff,
                    double t_ref, double t_absmax, int npt, const double *k, int nkc, const double *t0,
                    int ldt0, int nep, const double *p, const double *a, const double *inc, const double *e,
                    const double *w, int npv, int nlc, int npb, const int32_t *lcids, const int32_t *pbids,
                    const int32_t *epids, const int32_t *nsamples, const double *exptimes, const float *ldp,
                    const float *istar, const float *weights, int nk, int ng, int nz, double dk, double kmin,
                    double kmax, double dg, const double *z_edges, const double *obs, const double *sigma,
                    void *workspace, size_t workspace_bytes, double *lnl, double *grad, void *stream);

/* ---- independent cross-check: the Mandel & Agol quadratic model ----------- */

/* Flux of a star with quadratic limb darkening (u1, u2) occulted by a disk of
 * radius ratio k at the centre distances z[n], FP64: eval_quad_z_s
 * (pytransit/models/numba/ma_quadratic_nb.py:277-389; Mandel & Agol 2002,
 * complete elliptic integrals by Abramowitz & Stegun 17.3.34/36 and Bulirsch's
 * iteration for the third kind). */
int rr_ma_quad_z_f64(const double *z, int n, double k, double u1, double u2, double *flux, void *stream);
/* The quadratic model on the RoadRunner orbit layer: with a workspace from
 * rr_prepare_f64 (Taylor coefficients, contact points) and the arguments of
 * rr_flux_f64, the same phase fold, z and bounding box, but the Mandel & Agol
 * flux per sample (quadratic_model_v, ma_quadratic_nb.py:532-597) with
 * ldc[npv, npb, 2].  Point by point against rr_flux_f64 this isolates the
 * RoadRunner discretisation (weight tables, interpolation). */
int rr_ma_quad_flux_f64(const double *times, int npt, const double *k, int nkc, const double *t0, int ldt0,
                        const double *p, int npv, int nlc, int npb, const int32_t *lcids, const int32_t *pbids,
                        const int32_t *epids, const int32_t *nsamples, const double *exptimes, const double *ldc,
                        const void *workspace, double *flux, int ldflux, void *stream);

/* ---- secondary eclipse ----------------------------------------------------- */

/* Workspace of rr_eclipse_f64 / rr_es_f64 (one record per parameter vector). */
size_t rr_eclipse_workspace_bytes(int npv);
/* eclipse_model (pytransit/models/roadrunner/model_eclipse.py:12-81), FP64: the
 * visible area of the planet disk, flux[npv, ldflux] = pi k^2 outside the
 * eclipse and the mean over the exposure samples of pi k^2 - A(1, k, z)
 * inside it; k[npv], t0[npv, ldt0] per epoch (epids[nlc]), rstar[npv] in
 * solar radii for the light travel time.  The orbit is expanded about
 * mid-eclipse (the mean-anomaly offset of orbits_py.eclipse_phase) and the
 * eclipse shifted by the light travel time across the orbit; invalid
 * parameter vectors give NaN rows. */
int rr_eclipse_f64(const double *times, int npt, const double *k, const double *t0, int ldt0, const double *p,
                   const double *a, const double *inc, const double *e, const double *w, const double *rstar,
                   int npv, int nlc, const int32_t *lcids, const int32_t *epids, const int32_t *nsamples,
                   const double *exptimes, void *workspace, size_t workspace_bytes, double *flux, int ldflux,
                   void *stream);
/* rr_eclipse_f64 with the fold (model_eclipse.py:70-72) once per 128-point
 * tile for the tiles that reach no box, from the FP64 tile summaries of
 * rr_time_tiles_f64: such a tile is pi k^2 at every point, the same bits as
 * rr_eclipse_f64. */
int rr_eclipse_f64_culled(const double *times, const double *tiles64, int npt, const double *k, const double *t0,
                          int ldt0, const double *p, const double *a, const double *inc, const double *e,
                          const double *w, const double *rstar, int npv, int nlc, const int32_t *lcids,
                          const int32_t *epids, const int32_t *nsamples, const double *exptimes, void *workspace,
                          size_t workspace_bytes, double *flux, int ldflux, void *stream);
/* esmodel (model_ecspec.py:13-63), FP64: flux[npv, npb, ldflux] for the flux
 * ratios fratio[npv, npb], one zero epoch t0[npv], nsamples0 / exptime0. */
int rr_es_f64(const double *times, int npt, const double *k, const double *t0, const double *p, const double *a,
              const double *inc, const double *e, const double *w, const double *rstar, const double *fratio,
              int npv, int npb, int nsamples0, double exptime0, void *workspace, size_t workspace_bytes,
              double *flux, int ldflux, void *stream);
/* Split precision of the two (same models, same arguments as the FP64 entry
 * points, FP32 output): times_ff / t_ref / t_absmax from rr_time_split; the
 * FP64 per-pv prologue (eclipse shift, light travel time, Taylor jet) is
 * rounded to FP32 records; each point's time is folded exactly in FP32 pairs
 * and its samples are evaluated in FP32.  Tiles of 128 points whose time
 * range reaches no eclipse window are runs of stores of pi k^2 (eclipse) or 1
 * (ES).  rr_es_split treats every point as one light curve (nsamples0,
 * exptime0), as esmodel does. */
size_t rr_eclipse_split_workspace_bytes(int npv, int nlc, int npb);
int rr_eclipse_split(const float *times_ff, double t_ref, double t_absmax, int npt, const double *k,
                     const double *t0, int ldt0, const double *p, const double *a, const double *inc,
                     const double *e, const double *w, const double *rstar, int npv, int nlc, const int32_t *lcids,
                     const int32_t *epids, const int32_t *nsamples, const double *exptimes, void *workspace,
                     size_t workspace_bytes, float *flux, int ldflux, void *stream);
int rr_es_split(const float *times_ff, double t_ref, double t_absmax, int npt, const double *k, const double *t0,
                const double *p, const double *a, const double *inc, const double *e, const double *w,
                const double *rstar, const double *fratio, int npv, int npb, int nsamples0, double exptime0,
                void *workspace, size_t workspace_bytes, float *flux, int ldflux, void *stream);

/* ---- sampler parameter mapping -------------------------------------------- */

/* BaseLPF.transit_model's parameter mapping (pytransit/lpf/lpf.py:435-443) on
 * the device: pv[npv, ldpv] rows [tc, p, rho, b, k2, q1, q2 per passband from
 * column ld_start] -> k = sqrt(k2), t0 = tc - tref, p, a = as_from_rhop(rho, p)
 * (pytransit/orbits/orbits_py.py:604-618), i = i_from_ba(b, a)
 * (orbits_py.py:674-689), ldc[npv, npb, 2] = map_ldc(q) (lpf.py:85-91). */
int rr_lpf_map(const double *pv, int npv, int ldpv, int npb, int ld_start, double tref, double *k, double *t0,
               double *p, double *a, double *inc, double *ldc, void *stream);

/* ---- stated error bounds of the split paths ----------------------------------- */

/* No counterpart in the reference (the reference has one precision): after
 * rr_prepare_split[_ld] (resp. rr_ts_prepare_split[_ld]) on `workspace`, an
 * upper bound of |F_split - F_FP64| over all points of each parameter vector,
 * bound[npv] (FP64, 0 for an invalid vector), and their maximum in
 * *bound_max if not NULL.  p, a, inc, e, w are the same FP64 parameters. */
int rr_split_error_bounds(const double *p, const double *a, const double *inc, const double *e, const double *w,
                          int npv, int npb, int nlc, int nep, int ng, double dg, const void *workspace,
                          double *bound, double *bound_max, void *stream);
int rr_ts_split_error_bounds(const double *p, const double *a, const double *inc, const double *e, const double *w,
                             int npv, int npb, int ng, double dg, int nsamples0, double exptime0,
                             const void *workspace, double *bound, double *bound_max, void *stream);

/* ---- serving: many requests in one persistent launch ---------------------- */

/* One request of the serving loop (all pointers on the device).
 * kind 0, a RoadRunner request: the data of rr_time_split (times_ff) and
 * set_data (lcids), the tables written by rr_prepare_split
 * (rr_full_split_tables gives their addresses inside the workspace) and the
 * output flux[npv, ldflux].
 * kind 1, a transmission-spectroscopy request: times_ff, the tables written by
 * rr_ts_prepare_split[_ld] (rr_ts_tables: orb32 <- the per-pv records, lc32 <-
 * the channel records, ldm <- the LD means), npb channels, nsamples0,
 * exptime0 and dg, and the output flux[npv, npb, ldflux]; lcids and nlc are
 * not used. */
typedef struct {
  const float *times_ff;
  const int32_t *lcids;
  const float *orb32;
  const float *lc32;
  const float *ldm;
  float *flux;
  int64_t ldflux;
  int32_t npt, npv, nlc, npb, ng, kind;
  float inv_dg, exptime0;
  double dg;
  int32_t nsamples0, pad;
} rr_serve_request;

/* A unit of work: parameter vectors [pv0, pv1) x 128-point tiles [tile0, tile1) of request req. */
typedef struct {
  int32_t req, pv0, pv1, tile0, tile1, pad;
} rr_serve_item;

/* sizeof(rr_serve_request), sizeof(rr_serve_item) (for bindings that build the arrays) */
void rr_serve_struct_sizes(int *request_size, int *item_size);
void rr_full_split_tables(void *workspace, int npv, int npb, int nlc, int nep, int ng, const float **orb32,
                          const float **lc32, const float **ldm);
/* No counterpart in the reference (serving layer): nblocks persistent blocks
 * take the items items[0 .. *nitems) from *counter (set to 0 beforehand) and
 * write every covered flux value of the requests (every channel row of a
 * transmission-spectroscopy request; its items span at most 32 tiles);
 * returns at launch. */
int rr_serve_flux_split(const rr_serve_request *reqs, const rr_serve_item *items, const int *nitems, int *counter,
                        int nblocks, void *stream);

/* The set-up of one served request (no counterpart in the reference): every
 * field is 8 bytes.  stage -> dst (n_in bytes) is the host-to-device copy of
 * the request's inputs (stage in pinned memory); the other pointers are
 * device addresses of those inputs and of the request's own tables (times_ff,
 * ldp/istar for RoadRunner, ws, bnd[npv], bmax) and output; mu, basis,
 * weights, z_edges are the model's tables; desc (pinned, may be NULL) receives
 * the request's descriptor for rr_serve_flux_split, bound_host (pinned, may
 * be NULL) its stated error bound. */
typedef struct {
  const void *stage;
  void *dst;
  int64_t n_in;
  const double *time;
  const int32_t *lcids, *pbids, *epids, *nsamples;
  const double *exptimes, *k, *t0, *p, *a, *inc, *e, *w, *ldc;
  float *times_ff, *ldp, *istar;
  void *ws;
  double *bnd, *bmax;
  float *flux;
  const double *mu;
  const float *basis, *weights;
  const double *z_edges;
  int64_t npt, npv, nlc, npb, nep, nkc, npar, law, nb, nk, nz, ng, ldflux, wsb, nsamples0;
  double t_ref, t_abs, dk, kmin, kmax, dg, exptime0;
  double *bound_host;
  rr_serve_request *desc;
} rr_serve_setup_args;
/* kind 0: RoadRunner (rr_time_split, rr_prepare_split_ld, rr_split_error_bounds);
 * kind 1: transmission spectroscopy (rr_time_split, rr_ts_prepare_split_ld,
 * rr_ts_split_error_bounds); all enqueued on stream. */
int rr_serve_setup(int kind, const rr_serve_setup_args *args, void *stream);
void rr_serve_setup_args_size(int *size);

/* ---- no-allocation variant ------------------------------------------------- */

/* No counterpart in the reference: an addition for callers that cannot
 * allocate GPU memory themselves (a plugin host that owns the device and
 * passes a plugin only its inputs and outputs, a pool-based runtime that
 * forbids raw cudaMalloc, or a latency-bound loop where cudaMalloc's possible
 * device synchronisation is not acceptable).
 *
 * Same model and arguments as rr_full_split, without the workspace: the
 * per-parameter-vector tables live in a fixed file-scope device array of
 * rr_full_split_noalloc_max_bytes() bytes (32 MiB) that every GPU loading the
 * library holds until process exit.  The caller still passes inputs and
 * outputs.  Returns RR_ERR_WORKSPACE, before launching anything, when
 * rr_full_split_workspace_bytes(npv, npb, nlc, nep, ng) exceeds that size.
 * It calls no cudaMalloc/cudaFree.  The first call on a device looks up the
 * array's device address (cudaGetSymbolAddress) with that device current;
 * make that first call before any stream capture.  The address is kept per
 * device and CUDA context: the first call after a device reset (a new
 * context) looks it up again.  All calls share the one
 * array, which keeps the last call's contents (nothing in it needs clearing:
 * every table is written before it is read); calls that overlap on the GPU,
 * on different streams or host threads, race on it. */
size_t rr_full_split_noalloc_max_bytes(void);
int rr_full_split_noalloc(const float *times_ff, double t_ref, double t_absmax, int npt,
                          const double *k, int nkc, const double *t0, int ldt0, int nep,
                          const double *p, const double *a, const double *inc, const double *e,
                          const double *w, int npv, int nlc, int npb, const int32_t *lcids,
                          const int32_t *pbids, const int32_t *epids, const int32_t *nsamples,
                          const double *exptimes, const float *ldp, const float *istar,
                          const float *weights, int nk, int ng, int nz, double dk, double kmin,
                          double kmax, double dg, const double *z_edges, float *flux, int ldflux,
                          void *stream);

#ifdef __cplusplus
}
#endif

#endif /* PYTRANSIT_GB300_H */
