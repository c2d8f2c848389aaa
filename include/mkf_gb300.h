/*
 * mkf_gb300.h -- C ABI of the GB300 (sm_103a) filtering hot path of the
 * mkfbodytracker_pdaf upper-body tracker.
 *
 * One shared library (libmkf_gb300.so) exports every function below.  All
 * signatures use plain pointers, sizes and POD structs; device pointers are
 * named d_*, host pointers have no prefix.  Every call that touches the GPU
 * takes a stream (a cudaStream_t passed as mkf_stream_t; NULL = legacy default
 * stream).  Every function returns an MKF_* status; no exception or C++ type
 * crosses the ABI.  A handle is single-stream and not thread-safe; distinct
 * handles are independent (the reference's filters are likewise driven from
 * one ROS spin thread, pfPoseTracker.cpp:11).
 *
 * Randomness: the reference draws from cv::RNG(getTickCount()) per resample
 * (pf2DRao.cpp:179), cv::theRNG in randn (pf2DRao.cpp:96) and rand()
 * (pf2D.cpp:228,255), so its runs are not reproducible.  Here every draw is
 * Philox4x32-10 keyed by (seed, track) and counted by (frame, item, stream),
 * or an explicit uniform passed by the caller, so CPU and GPU see the same
 * draws.  Layout of one particle-frame's draws: ceil(d/4) Philox blocks at
 * streams 0..; words 2p,2p+1 give Box-Muller pair p from their top 23 bits
 * (u1 = 1 - (w0 >> 9) 2^-23, u2 = (w1 >> 9) 2^-23); the component uniform is
 * the 24-bit value of the low bytes of words 0..2, shifted right by one, times
 * 2^-23.  Resampling uniform of
 * frame f: word 0 of block (f, 0xFFFFFFFF, 0x100).  Prior draws use frame
 * 0xFFFFFFFF.
 */
#ifndef MKF_GB300_H
#define MKF_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* mkf_stream_t;   /* == cudaStream_t */

enum {
  MKF_OK = 0,
  MKF_ERR_ARG = 1,       /* bad argument / size out of range */
  MKF_ERR_CUDA = 2,      /* a CUDA runtime call failed (message in mkf_last_error) */
  MKF_ERR_NONPD = 3,     /* innovation covariance not positive definite */
  MKF_ERR_NAN = 4,       /* NaN/Inf produced */
  MKF_ERR_TIMEOUT = 5,   /* a bounded device wait gave up */
  MKF_ERR_NOMEM = 6,     /* allocation failed */
  MKF_ERR_STATE = 7      /* call out of order (e.g. update before reset) */
};

/* per-track / per-filter status bits (returned in status arrays) */
enum {
  MKF_ST_FALLBACK = 1,   /* a resampling step took the max-weight-0 fallback
                            (pf2DRao.cpp:184-192) */
  MKF_ST_NAN = 2,        /* a NaN/Inf log-likelihood was seen */
  MKF_ST_NONPD = 4,      /* an innovation covariance was not positive definite */
  MKF_ST_TRUNC = 8       /* a detection list longer than MKF_MAX_DET was truncated */
};

#define MKF_MAX_D 24       /* state dimension (PCA dims) */
#define MKF_MAX_K 32       /* mixture components */
#define MKF_MAX_J 4        /* measured joints */
#define MKF_MAX_DET 16     /* detections per joint list */
#define MKF_MAX_M 8        /* RBPF measurement rows */

const char* mkf_version(void);
/* message of the last failing call on this thread ("" if none) */
const char* mkf_last_error(void);

/* ------------------------------------------------------------------ K1 draws */
/* Host Philox4x32-10 block: key = {lo32(seed), hi32(seed) ^ track},
 * ctr = {frame, item, stream, 0}. */
int mkf_philox_block(uint64_t seed, uint32_t track, uint32_t frame, uint32_t item,
                     uint32_t stream, uint32_t out[4]);
/* The exact per-particle draws the particle kernels use for items 0..n-1 of
 * one frame: d_eps (n*d normals, row per particle), d_ucomp (n component
 * uniforms).  Replaces randn (pf2DRao.cpp:96) / pf2D.cpp:151-153. */
int mkf_draw_particles(uint64_t seed, uint32_t track, uint32_t frame, int n, int d,
                       float* d_eps, float* d_ucomp, mkf_stream_t stream);

/* ------------------------------------------------------- A6 systematic resample */
/* ParticleFilter::resample(weights, N) (pf2DRao.cpp:175-210).  Weights are
 * quantised to 64-bit integers with 40 bits below the largest (exact power-of-
 * two scaling, truncation) and resampled exactly: idx[i] = first j with
 * Q_j >= (i + U/2^32) Q_{L-1} / N (ties to the lower index, as the wheel's
 * strict '>').  All-zero/NaN weights take the reference's uniform-random
 * fallback (pf2DRao.cpp:184-192) with idx_i = floor(u_i L),
 * u_i = Philox(key {U, 0x5EED}, ctr {i,0,0,0}).  d_fallback (optional, one int)
 * receives 1 if the fallback was taken.  L, N <= 2^23. */
int mkf_resample_f64(const double* d_w, int L, int N, uint32_t U, int* d_idx,
                     int* d_fallback, mkf_stream_t stream);
int mkf_resample_f32(const float* d_w, int L, int N, uint32_t U, int* d_idx,
                     int* d_fallback, mkf_stream_t stream);
/* Allocation-free variant of mkf_resample_f32 (no counterpart in the reference,
 * whose resampler is host code).  For callers that must not allocate device
 * memory, e.g. a per-frame loop that cannot afford cudaMalloc's implicit device
 * synchronisation or an application that budgets its device memory up front:
 * the scratch is a fixed array inside the library (about 2 KB per GPU, held
 * until exit), so L must not exceed 1048576 weights (MKF_ERR_ARG otherwise).
 * The first call on each device looks up the array's device address, so make
 * that first call before any stream capture.  All calls share the one array:
 * calls that can overlap on the GPU (different streams) race and must be
 * serialised by the caller. */
int mkf_resample_f32_noalloc(const float* d_w, int L, int N, uint32_t U, int* d_idx,
                             int* d_fallback, mkf_stream_t stream);

/* ------------------------------------------- A1/A13 mixture-of-MRRW motion model */
/* Stacked per-model arrays (leading dimension n_models), all host pointers.
 * Config form of my_gmm::loadGaussian (my_gmm.cpp:45-75): F_k = diag(a_k),
 * B_k = (I - A_k) mu_k, Q_k = Lq_k Lq_k^T, prior N(mu_k, S0_k S0_k^T), mixture
 * weights pi.  Measurement: joint j pixel = pinhole(Bm_j x + mm_j). */
typedef struct mkf_bpf_models {
  int n_models, d, K, J;
  const float* a;     /* n*K*d */
  const float* mu;    /* n*K*d */
  const float* Lq;    /* n*K*d(d+1)/2, packed lower row-major */
  const float* S0c;   /* n*K*d(d+1)/2 */
  const float* pi;    /* n*K (cumulated in float32, sequentially, by the library) */
  const float* Bm;    /* n*J*3*d */
  const float* mm;    /* n*J*3 */
  float fx, fy, cx, cy;
} mkf_bpf_models;

typedef struct mkf_bpf_track {
  int32_t n_particles;   /* 1 .. 2^22 (batched: 1 .. 8192) */
  int32_t n_frames;
  int64_t frame_base;    /* first global frame index of this track */
  uint64_t seed;
  uint32_t track_id;     /* Philox key component */
  int32_t model_index;
  float kappa;           /* clutter density, detections per px^2 (> 0) */
  float p_detect;        /* in (0, 1) */
  float sigma_px;        /* detection noise std, px */
} mkf_bpf_track;

/* ---- plain per-track bootstrap PF (pf2D ParticleFilter API, pf2D.h:25-51,
 * with the mixture motion model): construct / reset / update / estimate. */
typedef struct mkf_bpf* mkf_bpf_t;
int mkf_bpf_create(const mkf_bpf_models* models, const mkf_bpf_track* track, mkf_bpf_t* out);
/* prior draw x ~ N(mu_k, Sigma_k), k ~ pi (my_gmm::resetTracker, my_gmm.cpp:30-42) */
int mkf_bpf_reset(mkf_bpf_t h, mkf_stream_t stream);
/* one frame (pf2D.cpp:148-210 order: predict from the resampled set, weight,
 * estimate, resample).  d_det_off: J+1 offsets into d_det (x,y pairs).
 * Writes the frame's weighted-mean state (d), log-likelihood increment and ESS
 * to the optional device pointers. */
int mkf_bpf_update(mkf_bpf_t h, uint32_t frame, const int* d_det_off, const float* d_det,
                   float* d_est, float* d_loglik, float* d_ess, mkf_stream_t stream);
/* debug copies of the last update into caller device buffers (any may be NULL):
 * particles after propagation (SoA d x N), log-weights (N), normalised-to-max
 * weights (N; only filled while debug is enabled) and the ancestors drawn (N) */
int mkf_bpf_set_debug(mkf_bpf_t h, int enable);
int mkf_bpf_read_debug(mkf_bpf_t h, float* d_x, float* d_logw, float* d_w, int* d_anc,
                       mkf_stream_t stream);
int mkf_bpf_status(mkf_bpf_t h, int* status);
int mkf_bpf_destroy(mkf_bpf_t h);

/* Captured frame loop: n_frames consecutive mkf_bpf_update calls recorded once
 * into a CUDA graph (three kernel nodes per frame).  Frame t of a launch is
 * frame0 + t (frame0 given at launch, read on the device); its detections are
 * d_det_off + t*J (J+1 offsets into d_det), its outputs d_est + t*d,
 * d_loglik + t, d_ess + t (each may be NULL).  Buffers are bound at capture: a
 * launch reads what they hold when it runs, so a caller stages each chunk of
 * frames into the same buffers.  A launch is equivalent to the n_frames update
 * calls, and launches chain with each other and with mkf_bpf_update.  The
 * graph is valid while its filter exists. */
typedef struct mkf_bpf_graph* mkf_bpf_graph_t;
int mkf_bpf_graph_create(mkf_bpf_t h, int n_frames, const int* d_det_off, const float* d_det, float* d_est,
                         float* d_loglik, float* d_ess, mkf_bpf_graph_t* out);
int mkf_bpf_graph_launch(mkf_bpf_graph_t g, uint32_t frame0, mkf_stream_t stream);
int mkf_bpf_graph_destroy(mkf_bpf_graph_t g);

/* ---- batched uneven tracks: one persistent kernel over all tracks */
typedef struct mkf_bpf_batch* mkf_bpf_batch_t;
/* tracks: n_tracks descriptors; n_frames_total = sum of n_frames (global frame
 * index space); detections are per (global frame g, joint j) lists
 * det[det_off[g*J+j] .. det_off[g*J+j+1]).  The offsets are int32, so one run
 * holds at most 2^31 - 1 detections. */
int mkf_bpf_batch_create(const mkf_bpf_models* models, int n_tracks, const mkf_bpf_track* tracks,
                         int64_t n_frames_total, mkf_bpf_batch_t* out);
/* tuning: threads per CTA (64..512, multiple of 32) and CTAs per SM (0 = max);
 * default 256 threads, 3 CTAs per SM, variant VEC_LOADS | SEARCH | LOWSMEM.
 * Launch bounds of VEC_LOADS | SEARCH (with or without LOWSMEM): <= 256
 * threads at 2 CTAs per SM (3 when ctas_per_sm >= 3), 257..384 threads at 2,
 * 385..512 threads at 1; of the other variants: <= 256 threads at 2, 257..512
 * threads at 1.  Shared memory can bound residency further. */
int mkf_bpf_batch_set_tuning(mkf_bpf_batch_t h, int block_threads, int ctas_per_sm);
/* code variants (autotuned; applied to the d = 12 diagonal-noise model):
 * MKF_BPF_VEC_LOADS = float4 model loads, MKF_BPF_SEARCH = ancestors by binary
 * search over shared prefix sums (12 bytes/particle of shared memory) instead
 * of the scatter walk (8 bytes/particle), MKF_BPF_PAIR = two particles per
 * loop iteration (implies the other two), MKF_BPF_LOWSMEM = the search with
 * 8 bytes/particle of shared memory (ancestors behind a track's prefix sums
 * when 3 n_particles <= 2 x the batch's largest, else in global memory; needs
 * VEC_LOADS | SEARCH, not PAIR).  Results are identical. */
enum { MKF_BPF_VEC_LOADS = 1, MKF_BPF_SEARCH = 2, MKF_BPF_PAIR = 4, MKF_BPF_LOWSMEM = 8 };
int mkf_bpf_batch_set_variant(mkf_bpf_batch_t h, int flags);
/* device-resident run: outputs est (G*d), loglik (G), ess (G), status (n_tracks) */
int mkf_bpf_batch_run(mkf_bpf_batch_t h, const int* d_det_off, const float* d_det,
                      float* d_est, float* d_loglik, float* d_ess, int* d_status,
                      mkf_stream_t stream);
/* host-buffer run: copies detections in, runs, copies outputs out, synchronises.
 * n_det = number of (x,y) pairs in det.  The tracks run in the same
 * longest-first order as mkf_bpf_batch_run, in two launches: the first
 * grid-size tracks start once their own lists are copied, the rest after the
 * bulk copy.  Output buffers that are pinned and mapped (cudaHostAlloc, or
 * cudaHostRegister with cudaHostRegisterMapped) are written by the kernels
 * directly; others are staged on the device and copied after the run. */
int mkf_bpf_batch_run_host(mkf_bpf_batch_t h, const int* det_off, const float* det, int64_t n_det,
                           float* est, float* loglik, float* ess, int* status,
                           mkf_stream_t stream);
/* debug capture of one track's per-frame weights and ancestors (n_frames*N
 * each, device pointers; NULL disables) */
int mkf_bpf_batch_set_debug(mkf_bpf_batch_t h, int track, float* d_w, int* d_anc);
/* the persistent grid of the last run (SM count x resident CTAs per SM,
 * capped at n_tracks); 0 before the first run */
int mkf_bpf_batch_last_grid(mkf_bpf_batch_t h, int* grid);
int mkf_bpf_batch_destroy(mkf_bpf_batch_t h);


/* ---------------------------------------------- A12 legacy bootstrap PF (pf2D) */
/* pf2D's ParticleFilter(numParticles, numDims, side) with its my_gmm prior
 * (pf2D.h:12-51), FP64, literal semantics: update(z) weights each particle by
 * the GMM prior density (float expf, pf2D.cpp:157-164) times isotropic 2-D
 * Gaussians (variance 15) of columns 6,7 against z[0..1] and columns 0,1 against
 * z[2..3] (pf2D.cpp:168); normalises; resamples (exact systematic resampling
 * of the normalised weights; when every weight is 0 all columns are redrawn
 * uniformly over the constructor's ranges and the weights reset to 1/N,
 * pf2D.cpp:225-250); leaves the weights as they were otherwise (as the
 * reference does, so getEstimator weights the resampled particles with the
 * pre-resampling weights); then predicts: columns 0..7 += N(0, 5^2)
 * (pf2D.cpp:90-102; columns >= 8 get no noise).  Draws: column c uniform of
 * particle i from word c%4 of block (frame, i, 0x200 + c/4) (w / 2^32); the 8
 * normals from blocks (frame, i, 0x210..0x211) by Box-Muller; construction uses
 * frame 0xFFFFFFFF.  mean (K*d), cov (K*d*d), w (K): host; 8 <= d <= 32. */
typedef struct mkf_pf2d* mkf_pf2d_t;
int mkf_pf2d_create(int n_particles, int d, int side, int K, const double* mean, const double* cov,
                    const double* w, int width, int height, uint64_t seed, uint32_t track_id,
                    mkf_pf2d_t* out);
/* z: host, 4 doubles (head x, y; hand x, y) = the reference's 2x2 measurement */
int mkf_pf2d_update(mkf_pf2d_t h, uint32_t frame, const double* z, mkf_stream_t stream);
int mkf_pf2d_estimate(mkf_pf2d_t h, double* d_est, mkf_stream_t stream);
/* particles (N*d), weights (N), ancestors (N, -1 after a re-initialisation),
 * reinit (host int, optional: 1 if the last update re-initialised) */
int mkf_pf2d_read(mkf_pf2d_t h, double* d_particles, double* d_weights, int* d_anc, int* reinit,
                  mkf_stream_t stream);
/* the filter's own draws of one frame: 8 normals and d uniforms per particle */
int mkf_pf2d_draws(uint64_t seed, uint32_t track, uint32_t frame, int n, int d, double* d_eps,
                   double* d_u, mkf_stream_t stream);
int mkf_pf2d_destroy(mkf_pf2d_t h);

/* --------------------------------------- A1-A5, A7, A8, A10 Rao-Blackwellised PF */
/* pf2DRao ParticleFilter(int nParticles) + its my_gmm (pf2DRao.h:13-31,
 * my_gmm.h:20-33), FP64.  Each particle is a Kalman filter (state_params,
 * my_gmm.h:9-18) whose GMM component is redrawn every update by systematic
 * resampling of the mixture weights (pf2DRao.cpp:128).  Measurement model:
 * LINEAR (per component H_k x + BH_k, my_gmm.cpp:59-72) or PINHOLE (EKF per
 * particle: joint j pixel = pinhole(Bm_j x + mm_j), Jacobian at the
 * predicted state).  Particle tracks are independent copies after resampling
 * (the standard RBPF; the reference's shallow cv::Mat copy-assign at
 * pf2DRao.cpp:153-156 makes duplicates share buffers, which only the oracle
 * emulates). */
typedef struct mkf_rbpf* mkf_rbpf_t;
enum { MKF_MEAS_LINEAR = 0, MKF_MEAS_PINHOLE = 1 };
/* d in {12, 24}; m <= MKF_MAX_M measurement rows; K <= MKF_MAX_K components;
 * n_particles <= 65536 */
int mkf_rbpf_create(int d, int m, int K, int n_particles, int meas_mode, uint64_t seed,
                    uint32_t track_id, mkf_rbpf_t* out);
/* my_gmm::loadGaussian(u, s, H, m, w, g) (my_gmm.cpp:45-75), host pointers:
 * u (d), s (d*d), Hpca (d*F, the pca_proj matrix), mpca (F).  Sets F = g I,
 * B = (1-g) u, Q = (1-g^2) s, R = 100 I_6, H = H1 Hpca^T, BH = H1 mpca^T with the
 * head/hand/neck selector H1 of my_gmm.cpp:59-67 (requires m == 6, LINEAR). */
int mkf_rbpf_load_gaussian(mkf_rbpf_t h, int k, const double* u, const double* s,
                           const double* Hpca, const double* mpca, int F, double w, double g);
/* config form of a component: mu (d), a (d, F = diag(a)), Q (d*d), Sigma (d*d,
 * reset covariance), R (m*m), w; LINEAR additionally H (m*d), BH (m). */
int mkf_rbpf_set_component(mkf_rbpf_t h, int k, const double* mu, const double* a, const double* Q,
                           const double* Sigma, const double* R, double w, const double* H,
                           const double* BH);
/* PINHOLE geometry: Bm (J*3*d), mm (J*3) with J = m/2, camera intrinsics */
int mkf_rbpf_set_pinhole(mkf_rbpf_t h, const double* Bm, const double* mm, double fx, double fy,
                         double cx, double cy);
/* hand-pixel decode used by the PDAF association: LINEAR: hand = Hd x + hb with
 * Hd (2*d), hb (2) (rows 0,1 of H_pca^T x + m_pca, pfPose.cpp:222; pf2DRao.cpp:94);
 * PINHOLE: joint index `joint` of the pinhole geometry. */
int mkf_rbpf_set_hand_decode(mkf_rbpf_t h, const double* Hd, const double* hb, int joint);
/* my_gmm::resetTracker(bins) (my_gmm.cpp:30-42): track i <- (mu_bins[i],
 * Sigma_bins[i]).  bins (host, N) or NULL to draw bins = resample(pi, N) with
 * Philox uniform word 0 of block (0xFFFFFFFF, 0xFFFFFFFF, 0x102). */
int mkf_rbpf_reset(mkf_rbpf_t h, const int* bins, mkf_stream_t stream);
/* ParticleFilter::update(measurement) (pf2DRao.cpp:125-158): d_meas is N rows
 * of m values (the reference's m x N measurement, one column per particle);
 * mask selects the rows used.  Uniforms: indicators word 0 of block
 * (frame, 0xFFFFFFFF, 0x102), ancestors word 0 of (frame, 0xFFFFFFFF, 0x100). */
int mkf_rbpf_update(mkf_rbpf_t h, uint32_t frame, const double* d_meas, unsigned mask,
                    mkf_stream_t stream);
/* the same with explicit uniforms (U/2^32 in [0,1)) */
int mkf_rbpf_update_u(mkf_rbpf_t h, const double* d_meas, unsigned mask, uint32_t U_ind,
                      uint32_t U_anc, mkf_stream_t stream);
/* getEstimator() (pf2DRao.cpp:23-31): uniform mean of the tracks' states */
int mkf_rbpf_estimate(mkf_rbpf_t h, double* d_est, mkf_stream_t stream);
/* copies of the filter state / last update into caller device buffers (any may
 * be NULL): x (N*d), P (N*d*d), logw (N), normalised weights (N), indicators
 * (N), ancestors (N) */
int mkf_rbpf_read(mkf_rbpf_t h, double* d_x, double* d_P, double* d_logw, double* d_wn, int* d_ind,
                  int* d_anc, mkf_stream_t stream);
/* overwrite the tracks (device pointers x (N*d), P (N*d*d)) */
int mkf_rbpf_write(mkf_rbpf_t h, const double* d_x, const double* d_P, mkf_stream_t stream);
int mkf_rbpf_status(mkf_rbpf_t h, int* status);
int mkf_rbpf_destroy(mkf_rbpf_t h);

/* ------------------------------------------------------- A9 PDAF association */
/* PFTracker::getMeasurementProposal (pfPose.cpp:210-329) over a detection list,
 * for the two arm filters at once.  Per arm a: hat_a = the hand pixel decoded
 * from arm a's getEstimator(); each candidate c_j gets
 * w_j = Pa p_a(c_j) / (Pa p_a(c_j) + Pa p_o(c_j) + clutter (1 - 2 Pa)),
 * p = N(c; hat, var I2) with var = 0.8 * roi width (the covariance of
 * getSampleProb, pf2DRao.cpp:114); the weights are normalised and resampled
 * (mkf_resample semantics, uniform word 0 of block (frame, 0xFFFFFFFF, 0x103)
 * of that arm's key) into N bins, and measurement row i of arm a is
 * [head_x, head_y, c_bins[i].x, c_bins[i].y (, neck_x, neck_y if m == 6)] with
 * head = (x + w/2, y + h/2), neck = (x + w/2, y + 1.65 h) of the arm's ROI
 * (pfPose.cpp:303-323).  roi: host, 4 doubles per arm (x_offset, y_offset,
 * width, height).  d_cand: M candidate (x,y) pairs (device, M <= 65536); when
 * M == 0 the hand rows are not written (the caller masks them).  d_meas_a:
 * N*m per arm.  d_bins_a (optional): N per arm. */
int mkf_pdaf_associate(mkf_rbpf_t arm0, mkf_rbpf_t arm1, uint32_t frame, const double* roi,
                       const double* d_cand, int M, double Pa, double clutter, double* d_meas0,
                       double* d_meas1, int* d_bins0, int* d_bins1, mkf_stream_t stream);

/* ------------------------------------- f2 pose decode and 3-D back-projection */
/* For B estimates x (B*d, device): e = Hpca^T x + mpca (pfPose.cpp:347-348;
 * Hpca d*F row-major and mpca F, device) into d_e (B*F, optional), and the
 * get3Dpose back-projection (pfPose.cpp:93-127) into d_pos3d (B*15: per
 * estimate a 3x5 row-major matrix, columns hand, elbow, shoulder, head, neck;
 * optional, needs F >= 21): full state (u, v, Z) per joint at 0..14, yaw 15,
 * roll 16, pitch 17, t 18..20; R = R3(yaw) R2(pitch) R1(roll); P = Kc [R | t];
 * point = inv(P[:, 0:3]) ((u Z, v Z, Z) - P[:, 3]).  Kc: host 3x3 camera
 * matrix.  A singular P[:, 0:3] gives NaN points and sets MKF_ST_NONPD in
 * *d_status (device int).  1 <= d <= 24, 1 <= F <= 64. */
int mkf_pose_decode(const double* d_x, int B, int d, int F, const double* d_Hpca, const double* d_mpca,
                    const double* Kc, double* d_e, double* d_pos3d, int* d_status, mkf_stream_t stream);
/* publish2Dpos point record (pfPose.cpp:173-208) for B frames from both arms'
 * decoded vectors e1, e2 (B*F each, device): 8 (x, y) points per frame into
 * d_pts (B*16): hand1, hand2, head and neck (means of both arms), elbow1,
 * elbow2, shoulder1, shoulder2.  F >= 14. */
int mkf_pose2d_record(const double* d_e1, const double* d_e2, int B, int F, double* d_pts,
                      mkf_stream_t stream);

/* ------------------------------------ f1 likelihood-image measurement front end */
/* GaussianBlur(likelihood, 15 x 15, sigma 3, BORDER_DEFAULT) (pfPose.cpp:213)
 * of an 8-bit image (device, row pitch in bytes): separable, each pass the
 * fmaf chain over the taps w_k = exp(-(k-7)^2/18) / sum (double, rounded to
 * float) in tap order, reflect-101 border, then round-to-nearest-even and
 * saturate to 8 bits.  width, height >= 8; d_out must not alias d_in. */
int mkf_likelihood_blur(const uint8_t* d_in, int width, int height, int pitch_in, uint8_t* d_out,
                        int pitch_out, mkf_stream_t stream);
/* PFTracker::getMeasurementProposal over a (blurred) likelihood image
 * (pfPose.cpp:210-329) for both arms.  Per arm a, M candidates (10 N in the
 * reference): with init != 0 uniform in the box x in [max(x-4w, 0),
 * min(x+5w, W)), y in [min(y+h, H), min(y+7h, H)) of the arm's ROI (integer
 * bounds, pfPose.cpp:228-235), else hand_a + 0.8 w (n0, n1) (getSamples:
 * randn with the matrix 0.8 w I as its standard deviation, pf2DRao.cpp:85-103);
 * draws from Philox block (frame, j, 0x104) of the arm's key (words 0, 1:
 * uniforms w / 2^32, or a Box-Muller pair).  Weight of candidate c inside the
 * image (0 < x < W, 0 < y < H): L = like[int(y)][int(x)] / 255, w = 0 if
 * L == 0 else L / (Pa p_a(c) + Pa p_o(c) + clutter (1 - 2 Pa)) with
 * p = N(c; hand, 0.8 w I) (pfPose.cpp:250-289); outside: 0.  Then as
 * mkf_pdaf_associate: normalise, resample N bins, measurement rows.
 * d_cand_a (optional, M x 2 doubles) receive the candidates. */
int mkf_pdaf_propose_image(mkf_rbpf_t arm0, mkf_rbpf_t arm1, uint32_t frame, const double* roi,
                           const uint8_t* d_like, int width, int height, int pitch, int M, int init,
                           double Pa, double clutter, double* d_meas0, double* d_meas1, int* d_bins0,
                           int* d_bins1, double* d_cand0, double* d_cand1, mkf_stream_t stream);

/* ------------------------------------------- A11 mixture KF forward / adjoint */
/* Deterministic counterpart of ParticleFilter::update (pf2DRao.cpp:125-158):
 * per frame every component k predicts from the collapsed posterior
 * (x = a_k*x + (1-a_k)*mu_k, P = A_k P A_k + Lq_k Lq_k^T; my_gmm.cpp:53-58,
 * KF_model.cpp:11-15), runs sequential PDAF/EKF updates over the measured
 * joints (Bar-Shalom combined innovation; PDA weights as pfPose.cpp:247-298)
 * giving l_k = sum_j log[(1-P_D) kappa + P_D sum_i N(z_i; zhat, S)]; then
 * c_t = log sum_k pi_k exp(l_k), w_k = pi_k exp(l_k - c_t), moment-matched
 * collapse and symmetrisation of P.  logL = sum_t c_t (FP32 math, FP64 sums).
 * theta (flat, FP64) = [mu (K*d), a (K*d), Lq packed lower (K*d(d+1)/2), sigma];
 * pi and the prior covariances S0 are fixed.  The backward pass is a
 * hand-written reverse sweep with sqrt(T) checkpointing: the forward stores
 * the collapsed state every ceil(sqrt(T)) frames; the backward recomputes
 * each segment from its checkpoint and reverses it frame by frame.
 * Gradients are reduced across tracks in a fixed order (deterministic). */
typedef struct mkf_mixkf* mkf_mixkf_t;
typedef struct mkf_mix_model {
  int d, K, J;
  const double* pi;    /* K */
  const double* S0;    /* K*d*d */
  double fx, fy, cx, cy;
} mkf_mix_model;
/* tracks: n_frames, frame_base (global frame index), their bodies Bm
 * (n_tracks*J*3*d), mm (n_tracks*J*3), P_D and kappa; all host pointers.
 * d in {12, 24}, K <= 32, J <= 4. */
int mkf_mixkf_create(const mkf_mix_model* model, int n_tracks, const int* n_frames,
                     const int64_t* frame_base, const double* Bm, const double* mm,
                     const double* p_detect, const double* kappa, int64_t n_frames_total,
                     mkf_mixkf_t* out);
/* theta: host (mkf_mixkf_set_theta) or device (mkf_mixkf_set_theta_device) */
int mkf_mixkf_set_theta(mkf_mixkf_t h, const double* theta);
int mkf_mixkf_set_theta_device(mkf_mixkf_t h, const double* d_theta, mkf_stream_t stream);
int mkf_mixkf_theta_size(mkf_mixkf_t h);
/* forward: per-track logL (optional, n_tracks doubles) and the total (1 double),
 * device pointers; stores the checkpoints the backward pass needs */
int mkf_mixkf_forward(mkf_mixkf_t h, const int* d_det_off, const float* d_det, double* d_loglik,
                      double* d_total, mkf_stream_t stream);
/* backward: d logL_total / d theta into d_grad (theta-sized, device); needs the
 * checkpoints of a forward run with the current stride (MKF_ERR_STATE otherwise) */
int mkf_mixkf_backward(mkf_mixkf_t h, const int* d_det_off, const float* d_det, double* d_grad,
                       mkf_stream_t stream);
/* checkpoint stride C (frames per backward segment; C >= 1, or 0 for the
 * default: ceil(sqrt(T_max)), lowered when one segment's records of all
 * resident CTAs would not fit in 60 % of L2).  Gradients do not depend on C.
 * Run mkf_mixkf_forward again before the next backward. */
int mkf_mixkf_set_checkpoint_stride(mkf_mixkf_t h, int C);
int mkf_mixkf_checkpoint_stride(mkf_mixkf_t h);
int mkf_mixkf_status(mkf_mixkf_t h, int* status);
int mkf_mixkf_destroy(mkf_mixkf_t h);
/* one Adam step on device (maximising when maximize != 0):
 * m = b1 m + (1-b1) g; v = b2 v + (1-b2) g^2; theta +/-= lr mhat/(sqrt(vhat)+eps).
 * Entries with mask[i] == 0 (optional) are left unchanged. */
int mkf_adam_step(double* d_theta, const double* d_grad, double* d_m, double* d_v, const uint8_t* d_mask,
                  int n, int step, double lr, double b1, double b2, double eps, int maximize,
                  mkf_stream_t stream);

#ifdef __cplusplus
}
#endif
#endif
