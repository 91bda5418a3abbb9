/* madflow_gb300: C ABI of the GB300 (sm_103a) implementation of madflow's
 * leading-order integrand and its VEGAS integrator.
 *
 * Conventions
 *   - Every entry point returns an mf_status (0 = MF_OK); no C++ exception or
 *     abort crosses the ABI.  mf_status_string() names a code.
 *   - All array arguments are DEVICE pointers owned by the caller unless a
 *     parameter says "host".  Layouts are structure-of-arrays (SoA): an array
 *     documented as [a][b][N] holds element (i, j, event e) at
 *     ((i*b + j)*N + e).
 *   - `stream` is a cudaStream_t passed as void* (NULL = legacy default).
 *     Calls are asynchronous with respect to the host unless stated.
 *   - Handles are not shared between host threads without external locking;
 *     distinct handles may be used concurrently.  A handle owns scratch
 *     buffers that every call with it reuses (records, work counter, block
 *     partials): calls with one handle must not overlap on the GPU, so issue
 *     them on one stream or order the streams (events) between them.
 *
 * Particle order of g g > t t~ + (k-2) g is MadGraph's: 0, 1 incoming gluons,
 * 2 = t, 3 = t~, 4.. outgoing gluons.  Momenta are (E, px, py, pz), GeV.
 */
#ifndef MADFLOW_GB300_H
#define MADFLOW_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  MF_OK = 0,
  MF_ERR_ARG = 1,         /* invalid argument (null pointer, size, unsupported value) */
  MF_ERR_CUDA = 2,        /* a CUDA call failed; see mf_last_cuda_error() */
  MF_ERR_UNSUPPORTED = 3, /* process / precision not built */
  MF_ERR_CAPACITY = 4,    /* request exceeds a documented maximum */
  MF_ERR_NONFINITE = 5,   /* non-finite weights were produced (counted and zeroed) */
  MF_ERR_STATE = 6        /* the requested result does not exist yet */
} mf_status;

typedef enum { MF_PREC_FP64 = 0, MF_PREC_MIXED = 1 } mf_precision;
typedef enum { MF_NEWTON_BATCH = 0, MF_NEWTON_PER_EVENT = 1 } mf_newton_rule;

typedef struct mf_process mf_process;

const char* mf_version(void);
const char* mf_status_string(int status);
const char* mf_last_cuda_error(void);

/* ---- process handles ------------------------------------------------------
 * Replaces the generated module madflow's PyOut exporter writes
 * (madgraph_plugin/template_files/matrix_method_python.inc:56-138, the
 * Matrix_<proc> class): n_gluons = total number of gluons k (2: g g > t t~,
 * 3: ... g, 4: ... g g).  precision: MF_PREC_FP64 (all FP64) or MF_PREC_MIXED
 * (FP32 wavefunctions/vertices/colour sum; FP64 momenta, propagator
 * denominators and accumulation). */
int mf_process_create(int n_gluons, int precision, mf_process** out);
int mf_process_destroy(mf_process* proc);
/* nexternal, ncomb (helicity combinations), ncolor (colour flows), ndiags;
 * denominator = the helicity/colour average (matrix_method_python.inc:61-66). */
int mf_process_info(const mf_process* proc, int* nexternal, int* ncomb, int* ncolor, int* ndiags,
                    double* denominator);
/* host out[ncomb][nexternal] (PyOut_exporter.py:288-298 helicity table) */
int mf_process_helicities(const mf_process* proc, double* out);
/* host out[ncolor][ncolor], the colour matrix (PyOut_exporter.py:301-324) */
int mf_process_colour_matrix(const mf_process* proc, double* out);

/* Matrix_<proc>.smatrix(all_ps, mdl_MT, mdl_WT, GC_10, GC_11[, GC_12])
 * (matrix_method_python.inc:80-104; tests/mockup_debug_me.py:454-480).
 *   ps        [nexternal][4][N] FP64 momenta
 *   couplings [N or 1][3] complex as (re, im) pairs: GC_10, GC_11, GC_12;
 *             coupling_stride = 1 for per-event couplings (running alpha_s),
 *             0 for one shared set
 *   out       [N] |M|^2 summed over helicities and colours, averaged
 *   hel_out   optional [ncomb][N]: per-helicity values of Matrix_<proc>.matrix
 *             (matrix_method_python.inc:106-138), NULL to skip */
int mf_smatrix(const mf_process* proc, const double* ps, int64_t n_events, double mdl_MT, double mdl_WT,
               const double* couplings, int64_t coupling_stride, double* out, double* hel_out, void* stream);

/* ---- phase space (python_package/madflow/phasespace.py) -------------------
 * rambo (phasespace.py:145-212): x [4*n][N] uniforms, sqrts [N] (or one value
 * when sqrts_stride = 0), masses host [n] (NULL: massless); p [n][4][N], w [N].
 * newton_rule MF_NEWTON_BATCH reproduces phasespace.py:84-103 (the loop stops
 * for the whole batch when one event converges). */
int mf_rambo(const double* x, int64_t n_events, int n_particles, const double* sqrts, int64_t sqrts_stride,
             const double* masses, int newton_rule, double* p, double* w, void* stream);
/* ramboflow (phasespace.py:257-319), nparticles >= 4: x [4*(n-2)+2][N];
 * p [n][4][N], w [N], x1 [N], x2 [N]. */
int mf_ramboflow(const double* x, int64_t n_events, int n_particles, double com_sqrts, const double* masses,
                 int newton_rule, double* p, double* w, double* x1, double* x2, void* stream);
/* _boost_to_lab (phasespace.py:322-356), in place on p [n][4][N] */
int mf_boost_to_lab(double* p, int64_t n_events, int n_particles, const double* x1, const double* x2, void* stream);

/* ---- external wavefunctions (python_package/madflow/wavefunctions_flow.py) -
 * p [4][N]; out [6][2][N] (slot, re/im, event), i.e. the reference's (6, N)
 * complex128 result.  sxxxxx returns 3 slots ([3][2][N]). */
int mf_ixxxxx(const double* p, int64_t n, double fmass, double nhel, double nsf, double* out, void* stream);
int mf_oxxxxx(const double* p, int64_t n, double fmass, double nhel, double nsf, double* out, void* stream);
int mf_vxxxxx(const double* p, int64_t n, double vmass, double nhel, double nsv, double* out, void* stream);
int mf_sxxxxx(const double* p, int64_t n, double nss, double* out, void* stream);

/* ---- ALOHA routines (tests/mockup_debug_me.py:43-397) ---------------------
 * wavefunctions [6][2][N]; coup host (re, im); amplitudes [2][N]. */
int mf_FFV1_0(const double* F1, const double* F2, const double* V3, const double* coup, int64_t n, double* out,
              void* stream);
int mf_FFV1_1(const double* F2, const double* V3, const double* coup, double M1, double W1, int64_t n, double* out,
              void* stream);
int mf_FFV1_2(const double* F1, const double* V3, const double* coup, double M2, double W2, int64_t n, double* out,
              void* stream);
int mf_VVV1P0_1(const double* V2, const double* V3, const double* coup, double M1, double W1, int64_t n,
                double* out, void* stream);

/* ---- integrand and VEGAS ---------------------------------------------------
 * Configuration of the integrand f(x, n_dim, weight) madflow hands to
 * vegasflow (scripts/madflow_exec.py:422-470; utilities.py:82-86).
 *   kind 0: g g > t t~ at fixed partonic sqrt(s): rambo over 8 uniforms,
 *           flux 389379365.6/(2 s) pb (phasespace.py:316-317);
 *   kind 1: hadronic: ramboflow (x1, x2 + rambo) at sqrt(S), synthetic gluon
 *           PDF luminosity f(x1) f(x2) / (x1 x2) at Q^2 = q2 (utilities.py:42-53),
 *           cuts on the outgoing gluons (pT > ptmin, |eta| < etamax,
 *           Delta R > drmin in the lab frame; <= 0 disables). */
typedef enum { MF_INITIAL_GG = 0, MF_INITIAL_PP = 1 } mf_initial_states;
/* One cut of madflow's PhaseSpaceGenerator.register_cut(variable, particle,
 * min_val, max_val) (phasespace.py:405-478): the variable of one particle
 * (MadGraph order, 0 .. nexternal-1) on the momenta before the boost to the
 * lab frame, kept when min_val < value (has_min) and value < max_val
 * (has_max), the thresholds held through float32 as madflow's float_me holds
 * them.  pt = sqrt(px^2 + py^2), mt2 = p.p + pt^2, mt = sqrt(mt2) (madflow's
 * three), eta = artanh(pz / |p|) (an addition). */
#define MF_MAX_CUTS 8
typedef enum { MF_CUT_PT = 0, MF_CUT_MT = 1, MF_CUT_MT2 = 2, MF_CUT_ETA = 3 } mf_cut_variable;
typedef struct {
  int variable;
  int particle;
  int has_min, has_max;
  double min_val, max_val;
} mf_cut;
typedef struct {
  int kind;
  double sqrts;
  double mt, wt;
  double alpha_s;      /* couplings GC_10 = -g, GC_11 = i g, GC_12 = i g^2, g = 2 sqrt(pi alpha_s) */
  double ptmin, etamax, drmin;
  /* q2 > 0: fixed factorisation and renormalisation scale Q^2 = q2 (madflow's
   * --fixed_scale, scripts/madflow_exec.py:432-434), alpha_s fixed.
   * q2 < 0 (kind 1): madflow's default dynamical scale
   * (scripts/madflow_exec.py:428-431): per event mu^2 = (sum over the
   * outgoing particles of m_T / 2)^2, m_T^2 = p.p + p_T^2; the densities at
   * mu^2; alpha_s(mu^2) from one-loop running with five flavours from
   * alpha_s = alpha_s(M_Z^2), M_Z = 91.1876 GeV (the synthetic densities
   * carry no alpha_s of their own), entering |M|^2 per event as madflow's
   * per-event couplings do.  Otherwise (kind 1): MF_ERR_ARG. */
  double q2;
  int newton_rule;
  /* MF_INITIAL_GG: the g g process alone.  MF_INITIAL_PP (kind 1), as
   * madflow sums the processes of a run, each over its initial states and
   * their mirror images (scripts/madflow_exec.py:444-458, utilities.py:25-39),
   * with the synthetic quark densities (mf_pdf_xfx_flavour), q = d u s c:
   *   two gluons, p p > t t~: f = weight x [L_gg |M|^2(g g > t t~) +
   *     L_qq |M|^2(q q~ > t t~)], L_qq over (q, q~) and (q~, q);
   *   three gluons, p p > t t~ j: f = weight x [L_gg |M|^2(g g > t t~ g) +
   *     the channels q q~ > t t~ g, q g > t t~ q, q~ g > t t~ q~ and their
   *     mirror images (mf_smatrix_qq_ttxj)], the jet cuts on particle 4
   *     whatever its flavour.
   * Other multiplicities with MF_INITIAL_PP: MF_ERR_UNSUPPORTED. */
  int initial_states;
  /* > 0: mf_integrand, mf_vegas_iteration and mf_vegas_events run their
   * events in consecutive slices of at most events_limit events, as
   * vegasflow's VegasFlow(events_limit=...) hands the integrand one slice per
   * call (scripts/madflow_exec.py:474-487, config.py:121-176).  The handle's
   * scratch then holds two slices instead of the call (1.8 KB per event for
   * four gluons, mixed; mf_process_scratch_bytes): the phase space of the
   * next slice runs on a stream of the handle while the current slice's
   * matrix element runs on the caller's stream.  The batch Newton rule of
   * the massive phase space runs per slice, and the slices' sums add up in
   * results in slice order.  Uniforms and the per-event outputs do not
   * depend on the slicing.  0: one slice.  < 0: MF_ERR_ARG.  Stage timing
   * (mf_process_set_timing) records one-slice calls only. */
  int64_t events_limit;
  /* > 0 (kind 1): madflow's --pt_cut (scripts/madflow_exec.py:396-401,
   * phasespace.py:417-422, 458-466): p_T > ptmin_all, held through float32
   * as madflow's float_me holds it, for every outgoing particle, the tops
   * included; events failing it give 0.  It adds to the gluon cuts above.
   * <= 0: off.  With kind 0: MF_ERR_ARG. */
  double ptmin_all;
  /* cuts[0 .. ncuts-1] (kind 1), all of them applied beside the cuts above;
   * 0 <= ncuts <= MF_MAX_CUTS, a variable or particle out of range, or cuts
   * with kind 0: MF_ERR_ARG. */
  int ncuts;
  mf_cut cuts[MF_MAX_CUTS];
} mf_integrand_config;

/* Number of integration dimensions of a configuration (8 for kind 0,
 * 4*(n-2)+2 for kind 1). */
int mf_integrand_ndim(const mf_process* proc, const mf_integrand_config* cfg, int* ndim);

/* f(x): x [ndim][N] points of the unit hypercube -> f [N] (pb), 0 for events
 * failing the cuts (madflow_exec.py:466-468 scatters them back as zeros). */
int mf_integrand(const mf_process* proc, const mf_integrand_config* cfg, const double* x, int64_t n_events,
                 double* f, void* stream);

/* f(x) with x in rows, [N][ndim], madflow's xrand[N, ndim] layout
 * (madflow_exec.py:422), otherwise as mf_integrand.  x and f may each be
 * device memory or page-locked host memory (cudaHostAlloc /
 * cudaHostRegister): the kernels then read the points from, and write f to,
 * host memory directly (zero-copy over the host link, inside the call's
 * kernels, so no separate copy runs).  Other host memory: MF_ERR_ARG. */
int mf_integrand_rows(const mf_process* proc, const mf_integrand_config* cfg, const double* x, int64_t n_events,
                      double* f, void* stream);

/* One VEGAS iteration (Lepage, J. Comput. Phys. 27 (1978) 192), fused:
 * Philox4x32-10 uniforms (seed, stream id, iteration) -> grid map -> integrand
 * -> per-iteration sums.  grid [ndim][nbins+1] (device, the bin edges).
 * results (device) [2 + ndim*nbins]: sum of w = jac*f/N, sum of w^2, and per
 * bin sums of w^2 (the refinement weights).  f_out optional [N] (jac*f).
 * u_out optional [ndim][N] float32 copy of the uniforms.
 * The iteration index is read from the device int *iteration so a captured
 * CUDA graph can be replayed for successive iterations. */
int mf_vegas_iteration(const mf_process* proc, const mf_integrand_config* cfg, const double* grid, int nbins,
                       uint64_t seed, uint32_t stream_id, const int* iteration, int64_t n_events, double* results,
                       double* f_out, float* u_out, void* stream);

/* Several processes in one persistent launch (no counterpart in the reference,
 * which loops over its processes in Python, madflow_exec.py:444-455).
 * procs [nproc] distinct handles of one precision, nproc <= 4; batch j:
 * ps[j] [nexternal_j][4][n[j]] momenta (as mf_smatrix), out[j] [n[j]]
 * |M|^2.  Couplings coup [6] (GC_10, GC_11, GC_12 as re, im) and the top
 * mass and width are shared.  The events of all batches form one work list,
 * the process with the most colour flows first; blocks take events from a
 * global counter.  The colour sums run on the SIMT lanes. */
int mf_smatrix_multi(mf_process* const* procs, int nproc, const double* const* ps, const int64_t* n, double mt,
                     double wt, const double* coup, double* const* out, void* stream);

/* Event output (device-side events for an LHE writer; replaces the
 * per-iteration dump of lhe_writer.py:139-196, called from
 * madflow_exec.py:460-464).  One iteration of the fused pipeline at
 * `iteration` of the frozen grid, with, per event, f_out [N] = jac * f (0 for
 * events failing the cuts, as in mf_vegas_iteration) and ps_out
 * [N][nexternal][4] the lab-frame momenta (E, px, py, pz) madflow passes to
 * its writer (PhaseSpaceGenerator(com_output=False)); zero rows for events
 * failing the cuts.  The VEGAS event weight is f_out / N.  One channel only (an
 * event names its initial-state flavours): initial_states MF_INITIAL_GG, else
 * MF_ERR_UNSUPPORTED. */
int mf_vegas_events(const mf_process* proc, const mf_integrand_config* cfg, const double* grid, int nbins,
                    uint64_t seed, uint32_t stream_id, int iteration, int64_t n_events, double* f_out,
                    double* ps_out, void* stream);

/* Hit-or-miss unweighting on the device (replaces the MG5 lhe_parser
 * unweight call of lhe_writer.py:316-358): keep[e] = 1 when u_e * w_max <
 * |w_e|, u_e a Philox4x32-10 uniform of (seed, stream_id, event e), else 0.
 * w [N] device, keep [N] device bytes.  Kept events with |w| > w_max are
 * overweight (their relative weight is |w| / w_max). */
int mf_unweight(const double* w, int64_t n_events, double w_max, uint64_t seed, uint32_t stream_id,
                unsigned char* keep, void* stream);

/* Stage timing of the fused pipeline behind mf_integrand / mf_vegas_iteration
 * (no counterpart in the reference).  With timing enabled, each call records
 * CUDA events on its stream between its stages; mf_process_stage_ms then
 * gives, once the caller has synchronised that stream, the milliseconds of the
 * last call's MF_STAGES stages: [0] uniforms, grid map, massless phase space
 * and the batch Newton minimum, [1] massive correction + cuts + PDF +
 * matrix-element records, [2] matrix element, [3] accumulation.
 * Calls made while their stream is being captured into a CUDA graph record
 * nothing (MF_ERR_STATE until an uncaptured call has run). */
#define MF_STAGES 4
int mf_process_set_timing(mf_process* proc, int enable);

/* Autotuner of the matrix-element launch (no counterpart in the reference).
 * On the first call of mf_smatrix / mf_integrand / mf_vegas_iteration with at
 * least 262144 events that is not being captured into a CUDA graph, the
 * matrix-element kernel is timed with CUDA events on that call's own events
 * (up to 2^20) in MF_TUNE_VARIANTS variants -- colour sum on the SIMT lanes
 * (colour 0) or on the tensor cores (colour 1, FP32 processes with 24 or 120 colour
 * flows) x a grid of 1, 2, 4 or 8 waves of resident blocks -- and the fastest
 * is kept by the handle (that one call waits on the host for the timings).
 * Five-gluon processes (global workspace, fixed grid) tune only the colour
 * method, on 2^14 events, from 16384 events up.  MF_AUTOTUNE=0 in the
 * environment keeps the default
 * (colour 1 where available, 8 waves).  mf_process_tuning reports the
 * configuration, whether it was tuned, and (ms, optional, MF_TUNE_VARIANTS
 * floats) the time of each variant in milliseconds, index colour*4 +
 * log2(waves), -1 for variants that do not exist; mf_process_set_tuning
 * fixes a configuration (MF_ERR_UNSUPPORTED for tensor cores where there is
 * no such variant). */
#define MF_TUNE_VARIANTS 8
int mf_process_tuning(const mf_process* proc, int* colour, int* waves, int* tuned, float* ms);
int mf_process_set_tuning(mf_process* proc, int colour, int waves);

/* Device error flags the handle's kernels raised (no counterpart in the
 * reference): bit 0 = a bounded wait on the tensor cores ran out (the event
 * being evaluated and every later event of the same thread block got NaN in
 * out and hel_out; events that needed no work keep 0); bit 1 = non-finite
 * weights were replaced by 0 in an accumulation (see mf_process_nonfinite).
 * Synchronous device-to-host read; clear != 0 resets the flags. */
int mf_process_error_flags(mf_process* proc, int* flags, int clear);
/* Number of event weights jac * f of mf_vegas_iteration / mf_integrand /
 * mf_vegas_events calls that were not finite (NaN or +-inf, e.g. from
 * non-finite caller points) and entered the sums, the histogram and f_out as
 * 0, since the last clear (no counterpart in the reference, which would
 * carry the NaN into its integral).  Synchronous read; clear != 0 resets the
 * count.  Returns MF_ERR_NONFINITE when *count > 0, else MF_OK. */
int mf_process_nonfinite(mf_process* proc, int64_t* count, int clear);
/* Tries (~1 ms each) of every bounded wait of the matrix-element kernels on
 * the tensor cores before a thread block gives up (default 1000, about 1 s;
 * 0 <= tries <= 100000).  With tries = 0 the first wait of every block gives
 * up at once, which exercises the error path of bit 0 above without a GPU
 * fault: the block still waits (bounded, at the default limit) for its
 * tensor-core work to finish before it frees its tensor memory.  No
 * counterpart in the reference. */
int mf_process_set_wait_limit(mf_process* proc, int tries);
int mf_process_stage_ms(const mf_process* proc, float* ms);

/* Device bytes the handle holds as scratch of the fused pipeline and of
 * mf_smatrix (per-event records and state, sized to the largest slice or
 * call so far, block partials, the global workspace of five gluons); freed
 * by mf_process_destroy.  No counterpart in the reference (TensorFlow owns
 * its memory). */
int mf_process_scratch_bytes(const mf_process* proc, int64_t* bytes);

/* VEGAS accumulation for an integrand evaluated by the caller: f [N], jac
 * [N], bins [ndim][N] (from mf_vegas_sample); results (device)
 * [2 + ndim*nbins] as in mf_vegas_iteration, with w = f*jac*inv_n.
 * ndim * nbins <= 8192.  A bin index outside [0, nbins) adds to no bin (it
 * still counts in the sums of w and w^2).  Deterministic (fixed-order
 * reductions).  The block partials live in a buffer per host thread and
 * device, so calls of one thread on different streams must not overlap. */
int mf_vegas_accumulate(const double* f, const double* jac, const int32_t* bins, int64_t n_events, int ndim,
                        int nbins, double inv_n, double* results, void* stream);

/* mf_vegas_accumulate without any device allocation.  No counterpart in the
 * reference: it exists for callers that cannot call cudaMalloc, for instance
 * code that runs inside a region where allocation is forbidden (a timed or
 * captured section) or whose device memory belongs to a pool manager.  Same
 * arguments, kernels and results as mf_vegas_accumulate; the block partials
 * live in a fixed array inside the library (4.2 MB on every GPU that loads
 * it, held until the process exits).  Limit: ndim * nbins <= 2048, else
 * MF_ERR_CAPACITY.  The first call on each device resolves the array's device
 * address (cudaGetSymbolAddress) with that device current: make that first
 * call before any stream capture.  All calls share the array, so calls that
 * overlap on the GPU (concurrent streams, or several host threads) race:
 * serialise them. */
int mf_vegas_accumulate_noalloc(const double* f, const double* jac, const int32_t* bins, int64_t n_events, int ndim,
                                int nbins, double inv_n, double* results, void* stream);

/* Grid refinement of one iteration (device): grid [ndim][nbins+1] updated in
 * place from the per-bin weights hist [ndim][nbins] with damping alpha. */
int mf_vegas_refine(double* grid, const double* hist, int ndim, int nbins, double alpha, void* stream);

/* Stand-alone VEGAS map: u [ndim][N] -> x [ndim][N], jac [N], bins
 * [ndim][N] int32 (bit-exact bin indices for identical uniforms).  A uniform
 * outside [0, 1) is mapped through the nearest edge bin. */
int mf_vegas_sample(const double* grid, int ndim, int nbins, const double* u, int64_t n_events, double* x,
                    double* jac, int32_t* bins, void* stream);

/* Philox4x32-10 uniforms in (0,1): u [ndim][N] for events event0.. */
int mf_philox_uniforms(uint64_t seed, uint32_t stream_id, uint32_t iteration, uint64_t event0, int64_t n_events,
                       int ndim, double* u, void* stream);

/* Synthetic gluon PDF x g(x) = A x^-0.2 (1-x)^5 (A from the momentum sum rule
 * int x g dx = 1/2) on a 100 (log x) x 50 (log Q^2) table, bicubic lookup:
 * x [N], out [N]. */
int mf_pdf_xfx(const double* x, int64_t n, double q2, double* out, void* stream);
/* The synthetic density of flavour pdg (21 gluon; 1..4 d u s c; -1..-4 their
 * antiquarks), the same tables and lookup: x u_v = A x^0.5 (1-x)^3 (int u_v
 * = 2), x d_v = A x^0.5 (1-x)^4 (int d_v = 1), sea x qbar = A x^-0.2 (1-x)^7
 * with int x qbar = 0.03 (ubar, dbar), 0.015 (s = sbar), 0.005 (c = cbar),
 * u = u_v + ubar, d = d_v + dbar.  The reference reads LHAPDF grids through
 * pdfflow (scripts/madflow_exec.py:412-417); these stand in for them. */
int mf_pdf_xfx_flavour(int pdg, const double* x, int64_t n, double q2, double* out, void* stream);

/* q q~ > t t~ (the light-quark processes of p p > t t~; MadGraph's u u~ >
 * t t~ module: smatrix(all_ps, mdl_MT, mdl_WT, GC_11),
 * matrix_method_python.inc:80-104): ps [4][4][N] (q, q~, t, t~), couplings
 * as mf_smatrix (GC_11 is used), out [N] |M|^2 averaged over the initial
 * spins and colours.  precision MF_PREC_FP64 or MF_PREC_MIXED (FP32 spinors
 * and bilinears).  No scratch, no handle. */
int mf_smatrix_qq_ttx(int precision, const double* ps, int64_t n_events, double mdl_MT, double mdl_WT,
                      const double* couplings, int64_t coupling_stride, double* out, void* stream);

/* The light-quark processes of p p > t t~ j at leading order (MadGraph's
 * u u~ > t t~ g, u g > t t~ u, u~ g > t t~ u~ modules, five diagrams each):
 * channel 0: q(0) q~(1) > t(2) t~(3) g(4); 1: q(0) g(1) > t t~ q(4);
 * 2: q~(0) g(1) > t t~ q~(4).  ps [5][4][N], couplings as mf_smatrix (GC_10
 * and GC_11 are used), out [N] |M|^2 averaged over the initial spins and
 * colours (1/36, 1/96).  precision MF_PREC_FP64 or MF_PREC_MIXED (FP32
 * wavefunctions and amplitudes, FP64 propagator denominators).  The gluon
 * polarisations use madflow's float32 sqrt(1/2) (wavefunctions_flow.py:10).
 * No scratch, no handle; no counterpart in the reference's tests. */
int mf_smatrix_qq_ttxj(int precision, int channel, const double* ps, int64_t n_events, double mdl_MT,
                       double mdl_WT, const double* couplings, int64_t coupling_stride, double* out, void* stream);

/* ---- normalizing-flow importance sampler ---------------------------------
 * No counterpart in the reference (an addition of this implementation, used as
 * a VEGAS alternative).  Piecewise-quadratic coupling transform of one layer
 * (Mueller et al., ACM TOG 38 (2019) 145): x, y, u [N][nb] float32 values in
 * [0,1] of the nb transformed dimensions; params [N][nb][2K+1] float32 raw
 * bin widths (K) and vertex heights (K+1) from the conditioner network;
 * logdet [N] = sum over the nb dimensions of log pdf.  2 <= K <= 64.
 * mf_pq_forward: y = CDF(x); mf_pq_inverse: x = CDF^-1(u) (sampling);
 * mf_pq_backward: gradients of mf_pq_forward given dL/dy (gy, may be NULL)
 * and dL/dlogdet (glogdet, may be NULL) -> gx [N][nb], gparams like params. */
int mf_pq_forward(const float* x, const float* params, int64_t n, int nb, int K, float* y, float* logdet,
                  void* stream);
int mf_pq_inverse(const float* u, const float* params, int64_t n, int nb, int K, float* x, float* logdet,
                  void* stream);
int mf_pq_backward(const float* x, const float* params, const float* gy, const float* glogdet, int64_t n, int nb,
                   int K, float* gx, float* gparams, void* stream);
/* The same three kernels under the flow-sampler names of the boundary:
 * forward (density), inverse (sampling), gradient. */
int mf_flow_fwd(const float* x, const float* params, int64_t n, int nb, int K, float* y, float* logdet,
                void* stream);
int mf_flow_inv(const float* u, const float* params, int64_t n, int nb, int K, float* x, float* logdet,
                void* stream);
int mf_flow_grad(const float* x, const float* params, const float* gy, const float* glogdet, int64_t n, int nb, int K,
                 float* gx, float* gparams, void* stream);
/* One whole coupling layer of the sampling direction in one kernel on the
 * tensor cores (tcgen05, TF32 operands, FP32 accumulation): the conditioner
 * MLP na -> 64 -> 64 -> nb (2K+1) with ReLU, then the inverse transform of
 * the nb transformed dimensions.  z [N][dim] float32 points, updated in place
 * on the dimensions ib [nb] (device int32, clamped to [0, dim)); the MLP
 * reads the dimensions ia [na] (likewise) as 2 z - 1.  W1 [64][na], b1 [64], W2 [64][64], b2 [64], W3 [nb (2K+1)][64],
 * b3 [nb (2K+1)] in torch.nn.Linear layout (out x in); logq [N] += the sum of
 * log pdf.  1 <= na, nb <= 16, na + nb <= dim, K in {4, 8, 16},
 * nb (2K+1) <= 256.  err: device int set to 1 if a bounded tensor-core wait
 * ran out (the layer is then incomplete), 2 if the library was built without
 * the tensor-core instructions.  Needs an sm_103 GPU. */
int mf_flow_inv_layer_tc(float* z, int64_t n, int dim, const int* ia, int na, const int* ib, int nb, int K,
                         const float* W1, const float* b1, const float* W2, const float* b2, const float* W3,
                         const float* b3, float* logq, int* err, void* stream);
/* mf_flow_inv_layer_tc with BF16 GEMM operands (tcgen05 kind::f16, FP32
 * accumulation): the MLP inputs, weights and hidden activations rounded to
 * BF16 (to nearest even) where they enter a GEMM; biases, activations and the
 * transform in FP32.  Same arguments, limits and error flags.  The sampled
 * log density is that of the map as evaluated, so estimates stay unbiased. */
int mf_flow_inv_layer_tc_bf16(float* z, int64_t n, int dim, const int* ia, int na, const int* ib, int nb, int K,
                              const float* W1, const float* b1, const float* W2, const float* b2, const float* W3,
                              const float* b3, float* logq, int* err, void* stream);

/* Whole coupling layers in hand-written FP32 kernels (no counterpart in the
 * reference): the conditioner MLP na -> 64 -> 64 -> nb (2K+1) with ReLU (the
 * same weights and layouts as mf_flow_inv_layer_tc), then the transform of
 * the dimensions ib.  z_in, z_out [N][dim] float32 (may be the same array);
 * ia [na], ib [nb] device int32 dimension indices (clamped to [0, dim));
 * 1 <= na, nb <= 16, na + nb <= dim, K in {4, 8, 16}, nb (2K+1) <= 320;
 * logq [N] += the sum over ib of log pdf.
 * mf_flow_layer_density: y = CDF(x) on ib (the density direction of
 * training, NormalizingFlow.log_prob); mf_flow_layer_sample: x = CDF^-1(u)
 * (sampling, for shapes mf_flow_inv_layer_tc does not take). */
int mf_flow_layer_density(const float* z_in, float* z_out, int64_t n, int dim, const int* ia, int na, const int* ib,
                          int nb, int K, const float* W1, const float* b1, const float* W2, const float* b2,
                          const float* W3, const float* b3, float* logq, void* stream);
int mf_flow_layer_sample(const float* z_in, float* z_out, int64_t n, int dim, const int* ia, int na, const int* ib,
                         int nb, int K, const float* W1, const float* b1, const float* W2, const float* b2,
                         const float* W3, const float* b3, float* logq, void* stream);
/* Gradient of mf_flow_layer_density: z_in [N][dim] the layer's input,
 * g_out [N][dim] = dL/d(output), glogdet [N] = dL/d(the layer's log pdf
 * sum) -> g_in [N][dim] = dL/d(input) (not aliasing z_in or g_out) and the
 * weight gradients gW1 [64][na], gb1 [64], gW2 [64][64], gb2 [64],
 * gW3 [nb (2K+1)][64], gb3 [nb (2K+1)] (overwritten, not accumulated).
 * workspace: device scratch of at least mf_flow_layer_grad_workspace bytes
 * (the partial sums of up to one block per SM, summed in a fixed order, so
 * the gradient is reproducible). */
int mf_flow_layer_grad_workspace(int na, int nb, int K, int64_t* bytes);
int mf_flow_layer_grad(const float* z_in, const float* g_out, float* g_in, int64_t n, int dim, const int* ia, int na,
                       const int* ib, int nb, int K, const float* W1, const float* b1, const float* W2,
                       const float* b2, const float* W3, const float* b3, const float* glogdet, float* gW1, float* gb1,
                       float* gW2, float* gb2, float* gW3, float* gb3, float* workspace, int64_t workspace_bytes,
                       void* stream);

#ifdef __cplusplus
}
#endif
#endif
