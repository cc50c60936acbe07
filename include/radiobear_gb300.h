/*
 * radiobear_gb300 — C ABI of the GB300 (sm_103a) radioBEAR forward model.
 *
 * Plain C: opaque handle, plain pointers and sizes, int status codes, no
 * exceptions across the boundary.  The caller owns every buffer it passes;
 * the library owns the device memory behind a handle.  One handle per host
 * thread; calls on a handle are synchronous unless the name ends in
 * _device (those enqueue on the given CUDA stream and return).  Every call
 * on a handle is ordered after the work the handle's last _device call
 * enqueued (an event on that call's stream), so host calls and _device
 * calls on other streams may follow it at once; work captured into a CUDA
 * graph by the caller is not tracked: order its replays yourself.
 *
 * Units follow the reference: frequencies GHz, pressure bar, temperature K,
 * radii and path lengths km, absorption cm^-1 (dB/km when units_db = 1).
 * Frequencies lie in [0, 2e4] GHz and line centres in (0, 2e4] GHz (the
 * float32 line sums' range); others are rejected with RB_EINVAL.
 *
 * Reference interfaces each entry point replaces (paths relative to the
 * david-deboer/radiobear project root):
 *   rb_set_lines      the catalogue loaders readInputFiles of
 *                     radiobear/constituents/nh3/nh3_hs.py:62-67,
 *                     nh3/nh3_sjs.py:17-23, h2o/h2o_bk.py:17-62,
 *                     h2s/h2s_ddb.py:14-39, ph3/ph3_jh.py:18-61,
 *                     co/co_ddb.py:14-19
 *   rb_set_formalisms Alpha.setup_formalisms, radiobear/alpha.py:49-102
 *   rb_set_co_clouds  the other_dict entries Alpha.setup_formalisms copies
 *                     for co and clouds, radiobear/alpha.py:90-102
 *   rb_alpha          Alpha.get_layers / get_alpha_from_calc /
 *                     total_layer_alpha, radiobear/alpha.py:151-305, and the
 *                     per-gas plugins alpha(freq, T, P, X, P_dict, other_dict)
 *   rb_raypath        raypath.compute_ds, radiobear/raypath.py:108-273
 *   rb_brightness     Brightness.single, radiobear/brightness.py:30-126
 *   rb_forward        Planet.run's alpha_layers + b loop + bright_run,
 *                     radiobear/planet.py:59-160 (one call per spectrum set)
 *   rb_bright_run     Planet.run's b loop given Alpha.layers,
 *                     radiobear/planet.py:118-133, planet_base.py:244-274
 *   rb_atm_props      AtmosphereBase.computeProp, radiobear/atm_base.py:120-194
 *   rb_regrid         regrid.regrid (regridType = number of log-P steps or a
 *                     pressure grid), radiobear/regrid.py:11-176
 */
#ifndef RADIOBEAR_GB300_H
#define RADIOBEAR_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RB_ABI_VERSION 3

typedef struct rb_handle rb_handle;

/* status codes */
#define RB_OK 0
#define RB_EINVAL 1  /* bad argument (message in rb_last_error) */
#define RB_ECUDA 2   /* CUDA runtime error */
#define RB_ENOMEM 3  /* device allocation failed */
#define RB_ESTATE 4  /* call out of order (e.g. no lines uploaded) */

/* line families (rb_set_lines) and their column order */
#define RB_FAM_NH3_INV 0 /* fo, Io, Eo, gammaNH3o                (ammonia.npz) */
#define RB_FAM_NH3_ROT 1 /* fo_rot, Io_rot, Eo_rot, gNH3_rot, gH2_rot, gHe_rot */
#define RB_FAM_NH3_V2 2  /* fo_v2, Io_v2, Eo_v2 */
#define RB_FAM_NH3_SJS 3 /* f0, I0, E, G0                         (nh3.npz) */
#define RB_FAM_H2O 4     /* f_o, I_o, E_o, w_s, x_s, w_h2, w_he, x_h2, x_he, SR */
#define RB_FAM_H2S 5     /* f0, I0, E, GH2S                       (h2s.npz) */
#define RB_FAM_PH3 6     /* f0, I0, E, WgtI0, WgtFGB, WgtSB       (ph3jh + PH3WGT) */
#define RB_FAM_CO 7      /* f0, I0, E                             (co.npz, co_ddb) */

/* NH3 formalism (rb_set_formalisms) */
#define RB_NH3_OFF 0
#define RB_NH3_HS 1     /* nh3_hs */
#define RB_NH3_SJS 2    /* nh3_sjs */
#define RB_NH3_HS_SJS 3 /* nh3_hs_sjs pressure blend */
#define RB_NH3_DBS 4    /* nh3_dbs */
#define RB_NH3_DBS_SJS 5 /* nh3_dbs_sjs pressure blend */

/* co_ddb line shape (other_dict['coshape']); any other string is STD */
#define RB_COSHAPE_VOIGT 0 /* 'voigt': sum of Voigt shapes */
#define RB_COSHAPE_VVW 1   /* 'vvw': sum of Van Vleck-Weisskopf shapes */
#define RB_COSHAPE_DIFF 2  /* 'diff': Voigt minus VVW */
#define RB_COSHAPE_STD 3   /* pressure-blended shape times line strength */

/* clouds_idp particle switches (other_dict '<kind>' > 0), OR-ed */
#define RB_CLOUD_ICE 1     /* 'ice_p':    cloud H2O / 0.9, water dielectric */
#define RB_CLOUD_WATER 2   /* 'water_p':  cloud SOLN / 1.0, water dielectric */
#define RB_CLOUD_NH4SH 4   /* 'nh4sh_p':  cloud NH4SH / 1.2, n = 1.7 - 0.005i */
#define RB_CLOUD_NH3ICE 8  /* 'nh3ice_p': cloud NH3 / 1.6, n = 1.3 - 0.0001i */
#define RB_CLOUD_H2SICE 16 /* 'h2sice_p': cloud H2S / 1.5, n = 1.15 - 0.0001i */
#define RB_CLOUD_CH4 32    /* 'ch4':      cloud CH4 / 1.0, n = 1.3 - 0.00001i */

/* gas slots of per-gas outputs: the reference's sorted constituent order
 * of the line gases, then co and clouds */
#define RB_GAS_H2 0
#define RB_GAS_H2O 1
#define RB_GAS_H2S 2
#define RB_GAS_NH3 3
#define RB_GAS_PH3 4
#define RB_GAS_CO 5
#define RB_GAS_CLOUDS 6
#define RB_NGAS 7

/* rows of the layer composition array X[RB_NX][nL]: gas mole fractions,
 * then cloud densities (g/cm^3, the reference's cloud table columns) */
#define RB_X_H2 0
#define RB_X_HE 1
#define RB_X_CH4 2
#define RB_X_NH3 3
#define RB_X_H2O 4
#define RB_X_H2S 5
#define RB_X_PH3 6
#define RB_X_CO 7
#define RB_X_CL_H2O 8    /* cloud H2O (ice) */
#define RB_X_CL_SOLN 9   /* cloud SOLN (liquid water) */
#define RB_X_CL_NH4SH 10
#define RB_X_CL_NH3 11
#define RB_X_CL_H2S 12
#define RB_X_CL_CH4 13
#define RB_NX 14

/* geometry switches */
#define RB_GTYPE_ELLIPSE 0
#define RB_GTYPE_SPHERE 1
#define RB_LIMB_SHAPE 0
#define RB_LIMB_SEC 1

int rb_abi_version(void);
/* Last error message of the calling thread ("" if none). */
const char* rb_last_error(void);

/* Create a handle on CUDA device `device`. */
int rb_create(rb_handle** out, int device);
int rb_destroy(rb_handle* h);

/* Upload one line family.  cols is column-major: cols[c*n + i] is column c
 * of line i, columns in the order listed above.  Truncation by strength or
 * frequency is the caller's (the reference applies it in its loaders).
 * Lines are sorted by centre internally.  n = 0 clears the family. */
int rb_set_lines(rb_handle* h, int family, int n, int ncols, const double* cols);

/* Select formalisms: nh3 one of RB_NH3_*, the others 0/1;
 * h2state 'e' (equilibrium) or 'n' (normal) H2 for the CIA prefactor. */
int rb_set_formalisms(rb_handle* h, int nh3, int use_h2, int use_h2o, int use_h2s, int use_ph3,
                      int h2state);

/* co_ddb (co 0/1, coshape RB_COSHAPE_*) and clouds_idp (clouds 0/1,
 * cloud_mask of RB_CLOUD_*).  co_ddb needs RB_FAM_CO lines.  Both are off
 * after rb_create. */
int rb_set_co_clouds(rb_handle* h, int co, int coshape, int clouds, int cloud_mask);

/* Tiling of the absorption line sums (no reference counterpart: the
 * reference has no device decomposition).  M frequency slots per thread
 * (2 or 4), W warps per CTA (1..4), item_lines lines per work item
 * (multiple of 128).  Zeros select the automatic choice.  Takes effect at
 * the next call with new frequencies or catalogues; the autotuner
 * (radiobear_gb300.tune) drives it. */
int rb_set_alpha_tiling(rb_handle* h, int M, int W, int item_lines);

/* Launch shapes of the adjoint and scan kernels (no reference counterpart),
 * driven by the autotuner (radiobear_gb300.tune); 0 restores the automatic
 * choice.  RB_TUNE_JVP_FREQS: frequencies per CTA of the absorption JVP
 * (32, 64 or 128); RB_TUNE_JVP_CTAS: resident CTAs per SM it is compiled
 * for (256 threads: 3 or 4, default 3; 128 threads: 4, 5 or 6, default 5);
 * RB_TUNE_JVP_THREADS: threads
 * per CTA (128 or 256, a multiple of the frequencies per CTA; the threads
 * beyond the frequencies split the lines); RB_TUNE_SCAN_LANES:
 * frequency-pair lanes per (ray, chunk) item of the brightness scan (a
 * power of two in 4..128; a CTA of 128 threads takes 128 / lanes items).
 * RB_TUNE_ADJ_MODE: how the adjoint entry points get d alpha / d theta.
 * 1 (stored): the JVP runs before the scan, gives the scan's alpha and
 * stores d alpha / d theta (nL x nf x 20 bytes), contracted with
 * d loss / d alpha after the reverse sweep; 2 (recomputed): the forward
 * line sums give alpha and the JVP runs after the reverse sweep, contracting
 * as it goes (no per-frequency storage); 0 (automatic): stored when that
 * takes at most an eighth of the device memory. */
#define RB_TUNE_JVP_FREQS 1
#define RB_TUNE_JVP_CTAS 2
#define RB_TUNE_SCAN_LANES 3
#define RB_TUNE_JVP_THREADS 4
#define RB_TUNE_ADJ_MODE 5
int rb_set_tuning(rb_handle* h, int param, int value);

/* Absorption of nL layers at nf frequencies.
 *   P[nL] bar, T[nL] K, X[RB_NX][nL] composition (rows above), freqs[nf] GHz.
 *   scale:      nullable, [nL][RB_NGAS] multipliers (number, per-layer list
 *               and per-constituent dict scales of Alpha.get_layers all map
 *               onto this form).
 *   layers_out: nullable, [nf][nL]  total (Alpha.layers)
 *   gas_out:    nullable, [nL][nf][RB_NGAS] scaled per gas (Alpha.tosave)
 * units_db = 1 returns dB/km (the nh3_hs clamp then acts in dB/km). */
int rb_alpha(rb_handle* h, int nL, const double* P, const double* T, const double* X, int nf,
             const double* freqs, const double* scale, int units_db, double* layers_out,
             double* gas_out);

/* Ray paths of nb impact parameters b[nb][2] (fraction of R[0]).
 *   R[nL] equatorial layer radii (km, top first), N[nL] refractive index,
 *   Req/Rpol (km) set the shell ellipse and the aspect flattening,
 *   orient0/orient1 the orientation (deg), gtype/limb the switches above.
 * Outputs per ray: nseg[nb]; ds[nb][max_seg] km; layer[nb][max_seg];
 * nullable r4ds[nb][max_seg]; nullable latlng[nb][max_seg+1][2] (deg) of
 * each path point; nullable end_code[nb] (0 no path, 1 ran to the last
 * layer, 2 left the atmosphere, 3 max_seg too small).
 * max_seg >= 2*nL + 4 always suffices. */
int rb_raypath(rb_handle* h, int nL, const double* R, const double* N, double Req, double Rpol,
               double orient0, double orient1, int gtype, int limb, int nb, const double* b,
               int max_seg, int32_t* nseg, double* ds, int32_t* layer, double* r4ds,
               double* latlng, int32_t* end_code);

/* Brightness temperature of nb paths given absorption layers[nf][nL]
 * (cm^-1) and T[nL].  disc = 1 uses the 2 E2(tau) weighting of b = 'disc'.
 * Tb_out[nb][nf]; nullable intW_out[nb][nf]; nullable profiles
 * tau/W/TbL [nb][nf][max_seg] (entry 0 is the zero start value). */
int rb_brightness(rb_handle* h, int nL, const double* T, int nf, const double* layers, int nb,
                  const int32_t* nseg, const double* ds, const int32_t* layer, int max_seg,
                  int disc, double* Tb_out, double* intW_out, double* tau_out, double* W_out,
                  double* TbL_out);

/* The b loop of Planet.run (radiobear/planet.py:118-133 -> bright_run,
 * planet_base.py:244-274 -> Brightness.single, brightness.py:30-126) for nb
 * rays through one atmosphere at once, given the absorption the run already
 * computed: layers[nf][nL] (cm^-1, Alpha.layers), T[nL] K, R/N and the
 * geometry as in rb_raypath.  Ray paths stay on the device; the
 * absorption is uploaded once.  Exp weighting (the reference's 'disc' is a
 * single nadir ray: use rb_brightness with disc = 1).
 * Tb_out[nb][nf]; nullable intW_out[nb][nf]; nullable nseg_out[nb]
 * (0 for a ray that misses the planet, whose Tb is T_cmb). */
int rb_bright_run(rb_handle* h, int nL, const double* T, const double* R, const double* N,
                  double Req, double Rpol, double orient0, double orient1, int gtype, int limb,
                  int nf, const double* layers, int nb, const double* b, double* Tb_out,
                  double* intW_out, int32_t* nseg_out);

/* Fused forward model from host buffers: absorption, ray paths and Tb for
 * nb rays with device-resident intermediates.  Optional weights[nb] give
 * Tb_avg[nf] = sum_k weights[k] Tb[k][:].  disc = 1 evaluates every ray as
 * the reference's b = 'disc' (nadir, E2 weighting).
 * Outputs (all nullable): Tb_out[nb][nf], Tb_avg[nf], layers_out[nf][nL]. */
int rb_forward(rb_handle* h, int nL, const double* P, const double* T, const double* X,
               const double* R, const double* N, int nf, const double* freqs, const double* scale,
               double Req, double Rpol, double orient0, double orient1, int gtype, int limb,
               int nb, const double* b, const double* weights, int disc, double* Tb_out,
               double* Tb_avg, double* layers_out);

/* Same as rb_forward but every array argument is a device pointer, the
 * work is enqueued on `stream` (a cudaStream_t, 0 = legacy default) and the
 * call returns without synchronising.  Frequencies are planned from the
 * HOST array freqs_host (nf values) and cached on the handle.  disc = 1
 * applies the E2 weighting to the rays given (pass nadir rays for the
 * reference's b = 'disc'; device arrays are not rewritten). */
int rb_forward_device(rb_handle* h, void* stream, int nL, const double* P, const double* T,
                      const double* X, const double* R, const double* N, int nf,
                      const double* freqs_host, const double* scale, double Req, double Rpol,
                      double orient0, double orient1, int gtype, int limb, int nb,
                      const double* b, const double* weights, int disc, double* Tb_out,
                      double* Tb_avg);

/* Adjoint of the forward model (no reference counterpart: radioBEAR has
 * no derivatives).  Runs the forward and returns Tb, the weighted average
 * (when weights are given) and the gradient of
 *   loss = sum_f grad[f] Tb_avg[f]           (weights given, grad [nf])
 *   loss = sum_{b,f} grad[b][f] Tb[b][f]     (no weights, grad [nb][nf])
 * with respect to each layer's T (K), P (bar) and ln X of NH3, H2O, H2S:
 * dT[nL], dP[nL], dlnX[3][nL] (rows NH3, H2O, H2S).  The ray paths are
 * held fixed (they depend on R and N only); alpha is recomputed with its
 * layer derivatives instead of being stored.  disc = 0: exp weighting;
 * disc = 1: the b = 'disc' weighting 2 E2(tau) of brightness.py:96 on the
 * nadir ray (as rb_forward), differentiated with dE2/dx = -E1(x). */
int rb_adjoint(rb_handle* h, int nL, const double* P, const double* T, const double* X,
               const double* R, const double* N, int nf, const double* freqs, const double* scale,
               double Req, double Rpol, double orient0, double orient1, int gtype, int limb, int nb,
               const double* b, const double* weights, int disc, const double* grad,
               double* Tb_out, double* Tb_avg, double* dT, double* dP, double* dlnX);

/* Device-pointer variant of rb_adjoint (freqs on the host), enqueued on
 * `stream`; Tb_out and Tb_avg may be null.  disc = 1 applies the E2
 * weighting to the rays given (pass nadir rays for the reference's
 * 'disc'). */
int rb_adjoint_device(rb_handle* h, void* stream, int nL, const double* P, const double* T,
                      const double* X, const double* R, const double* N, int nf,
                      const double* freqs_host, const double* scale, double Req, double Rpol,
                      double orient0, double orient1, int gtype, int limb, int nb, const double* b,
                      const double* weights, int disc, const double* grad, double* Tb_out,
                      double* Tb_avg, double* dT, double* dP, double* dlnX);

/* Batches of atmospheres (no reference counterpart: the reference runs one
 * atmosphere per Planet): nvar variants, variant v with nL_host[v] layers
 * (HOST array).  P, T, R, N are the variants' [nL_v] arrays concatenated
 * (device, sum nL_v values), X is [RB_NX][sum nL_v] (device).  Every
 * variant uses the same nb impact parameters b[nb][2] and weights[nb]
 * (device); Tb_avg[nvar][nf] (device) receives the weighted averages.  All
 * variants run in the same launches (one persistent absorption launch over
 * every variant's layers, one ray-walk launch over all nvar nb rays, ...).
 * Frequencies are planned from the host array freqs_host.  scale
 * (nullable, device) is [sum nL_v][RB_NGAS]: per variant, per layer and
 * per gas multipliers, as rb_alpha's scale (the retrieval-reuse pattern of
 * scripts/demo_batch.py:24-41 with a scale dict per walker). */
int rb_forward_batch_device(rb_handle* h, void* stream, int nvar, const int32_t* nL_host,
                            const double* P, const double* T, const double* X, const double* R,
                            const double* N, int nf, const double* freqs_host, const double* scale,
                            double Req, double Rpol, double orient0, double orient1, int gtype,
                            int limb, int nb, const double* b, const double* weights,
                            double* Tb_avg);

/* Forward and adjoint of a batch: grad[nvar][nf] = d loss / d Tb_avg;
 * dT, dP [sum nL_v], dlnX [3][sum nL_v] (device). */
int rb_adjoint_batch_device(rb_handle* h, void* stream, int nvar, const int32_t* nL_host,
                            const double* P, const double* T, const double* X, const double* R,
                            const double* N, int nf, const double* freqs_host, const double* scale,
                            double Req, double Rpol, double orient0, double orient1, int gtype,
                            int limb, int nb, const double* b, const double* weights,
                            const double* grad, double* Tb_avg, double* dT, double* dP,
                            double* dlnX);

/* Number of this library's kernel launches made by the last rb_forward /
 * rb_forward_device call (for launch accounting). */
int rb_last_launch_count(rb_handle* h);

/* ---- atmosphere producer (gas / cloud column tables, float64) ----------
 * Tables are the reference's [ncol][n] column tables (n layers, pressure
 * increasing).  roles[4] = column indices of Z (km), T (K), P (bar), DZ
 * (cm); chem[3][ncol] = per column the molar mass (g/mol), c_p / R and the
 * microwave refractivity constant of chemistry.ConstituentProperties (a
 * negative refractivity selects the H2O law 245 + 1.28e6 / T); the role
 * columns are not constituents.  Property rows (RB_PROP_*) follow the
 * reference's LP order. */
#define RB_PROP_Z 0
#define RB_PROP_R 1      /* radius, km (Req at the layer nearest p_ref) */
#define RB_PROP_P 2
#define RB_PROP_GM 3
#define RB_PROP_AMU 4
#define RB_PROP_REFR 5
#define RB_PROP_N 6      /* refractive index */
#define RB_PROP_H 7
#define RB_PROP_LAPSE 8
#define RB_PROP_LAPSEP 9
#define RB_PROP_g 10
#define RB_NPROP 11
#define RB_ATM_MAXCOL 32

/* computeProp of one table: prop[RB_NPROP][nL] (host buffers). */
int rb_atm_props(rb_handle* h, int nL, int ncol, const int32_t* roles, const double* chem,
                 const double* gas, double Req, double p_ref, double GM_ref, double* prop);
/* computeProp of nvar tables concatenated along layers (device gas
 * [ncol][sum nL_v], prop [RB_NPROP][sum nL_v]), enqueued on `stream`. */
int rb_atm_props_device(rb_handle* h, void* stream, int nvar, const int32_t* nL_host, int ncol,
                        const int32_t* roles, const double* chem, const double* gas, double Req,
                        double p_ref, double GM_ref, double* prop);
/* regrid onto the increasing pressure grid Pgrid[nout]: linear in P inside
 * the table; deeper, constituents at their deepest value and T, Z along a
 * dry adiabat in hydrostatic equilibrium; above, T and Z along the last
 * slope; Z renormalised to 0 at the deepest point and DZ reset.  The cloud
 * table (nullable, same layers as the gas table, no chemistry) is
 * interpolated with 0 outside.  Host buffers; gas_out [ncol][nout],
 * cloud_out [ncl][nout]. */
int rb_regrid(rb_handle* h, int nin, int ncol, const int32_t* roles, const double* chem,
              const double* gas_in, int ncl, const int32_t* roles_cl, const double* cloud_in,
              int nout, const double* Pgrid, double Req, double p_ref, double GM_ref,
              double* gas_out, double* cloud_out);
/* Device form for nvar tables (layer counts nin_host, concatenated along
 * layers): every table onto nout points of its own grid pgrid + v *
 * pgrid_stride (stride 0: one shared grid); outputs [ncol][nvar * nout]
 * with table v at columns v * nout.  Enqueued on `stream`. */
int rb_regrid_device(rb_handle* h, void* stream, int nvar, const int32_t* nin_host, int ncol,
                     const int32_t* roles, const double* chem, const double* gas_in, int ncl,
                     const int32_t* roles_cl, const double* cloud_in, int nout, const double* pgrid,
                     int pgrid_stride, double Req, double p_ref, double GM_ref, double* gas_out,
                     double* cloud_out);

/* Phase timing.  With profiling on, rb_forward / rb_forward_device record
 * CUDA events around each kernel on the stream it is launched on;
 * rb_phase_times then fills ms[0..5] = layer prep, line sums, ray paths,
 * brightness, disc average, assembly of the absorption (first n of them)
 * of the last call (synchronises the handle). */
int rb_set_profiling(rb_handle* h, int on);
int rb_phase_times(rb_handle* h, double* ms, int n);

/* Float32 FMA throughput of the device (TFLOP/s), measured with probe
 * kernels (independent scalar FFMA chains and packed f32x2 FMA chains; the
 * higher rate is returned) at the current clocks: the roofline denominator
 * of the line sums. */
int rb_probe_fp32_peak(rb_handle* h, double* tflops);

/* Scratch limit of rb_brightness_noalloc: nb * ceil(max_seg / 128) * nf must
 * not exceed this many float4 elements (8 MiB, held by every GPU that loads
 * the library until the process exits). */
#define RB_NOALLOC_SCRATCH_ELEMS 524288

/* Brightness temperatures from device-resident inputs without allocating
 * device memory.  No counterpart in the reference: it exists for callers
 * that cannot call cudaMalloc -- applications that reserve all device
 * memory up front, plugins running inside a framework that owns the
 * allocator, real-time loops that forbid allocation (cudaMalloc/cudaFree can
 * synchronise the device and take unbounded time).
 * Every array is a device pointer on the calling thread's current device:
 *   alpha32[nL][nf] absorption (float32, cm^-1), T[nL] K, nseg[nb],
 *   ds[nb][max_seg] km, layer[nb][max_seg] (negative indices wrap as in
 *   Python, out-of-range indices are clamped), Tb[nb][nf] output.
 * The work is enqueued on `stream` (a cudaStream_t) and the call returns
 * without synchronising.  Its scratch is one fixed file-scope device array
 * shared by every call, so calls that overlap on the GPU race: serialise
 * them.  The first call on a device looks up that array's address; make it
 * before any stream capture.  That address is cached for the life of the
 * process: do not use this entry point after cudaDeviceReset (or another
 * reset of the device's primary context) on a device it has already run on.
 * Sizes beyond RB_NOALLOC_SCRATCH_ELEMS, and ceil(max_seg / 128) or
 * ceil(nf / 128) above 65535, are rejected with RB_EINVAL; nb itself is
 * limited only by the scratch size. */
int rb_brightness_noalloc(void* stream, int nL, int nf, const float* alpha32, const double* T,
                          int nb, const int32_t* nseg, const double* ds, const int32_t* layer,
                          int max_seg, double* Tb);

/* E2(x) evaluated by the device routine used for b = 'disc' (test hook). */
int rb_debug_e2(rb_handle* h, int n, const double* x, double* out);
/* E1(x) = -dE2/dx evaluated by the device routine of the disc adjoint
 * (test hook). */
int rb_debug_e1(rb_handle* h, int n, const double* x, double* out);

#ifdef __cplusplus
}
#endif
#endif /* RADIOBEAR_GB300_H */
