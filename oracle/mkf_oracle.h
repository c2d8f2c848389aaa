/*
 * mkf_oracle.h -- FP64 CPU restatement of the mkfbodytracker_pdaf filtering hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity reference for the CUDA product
 * (mkfbodytracker_pdaf_gb300/csrc) and the timed CPU baseline of bench.py; the
 * product never links, loads or calls it.
 *
 * Parity status: the reference (ROS + OpenCV, rosbuild) has no tests, golden
 * vectors or fixtures for this path, and its build needs ROS and OpenCV, which
 * are absent.  Its filter sources (KF_model.cpp, my_gmm.cpp, pf2DRao.cpp) are
 * compiled unmodified against stand-in OpenCV/ROS headers (oracle/refpin), and
 * their outputs (tests/golden/refpin.npz) pin the KF predict/update,
 * loadGaussian, the literal resampling wheel, the chol/mvnpdf quirk modes and
 * the literal RBPF update with its shared-buffer effect (tests/test_refpin.py).
 * Also pinned: Philox4x32-10 against the published Random123 known-answer
 * vectors, the exact systematic resampler against the literal wheel on dyadic
 * weights, and the KF / Gaussian restatements against closed forms.
 *
 * Every function cites the reference file:line it restates.
 */
#ifndef MKF_ORACLE_H
#define MKF_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- K1: Philox4x32-10 counter-based draws (replaces cv::RNG / randn / rand) */
void mko_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
/* key = {lo32(seed), hi32(seed) ^ track}, ctr = {frame, item, stream, 0} */
void mko_draw_block(uint64_t seed, uint32_t track, uint32_t frame, uint32_t item,
                    uint32_t stream, uint32_t out[4]);
float mko_u01_f32(uint32_t w);
/* Box-Muller normals for one particle-frame, d (even, <= 24) normals + 1
 * component uniform.  Layout: ceil(d/4) blocks at streams 0..; words 2p,2p+1
 * feed pair p with 23-bit uniforms u1 = 1 - (w >> 9) 2^-23, u2 = (w >> 9) 2^-23;
 * the component uniform is the 24-bit value of the low bytes of words 0..2,
 * shifted right by one, times 2^-23 (libm; the GPU uses its own intrinsics, so
 * parity tests feed GPU-dumped normals to the oracle instead of these). */
void mko_particle_draws(uint64_t seed, uint32_t track, uint32_t frame, uint32_t item,
                        int d, double* eps, float* ucomp);

/* ---- A6: systematic resampling (pf2DRao.cpp:175-210, pf2D.cpp:279-323) */
/* Literal reference wheel; u in [0,1); fallback[] used when max weight == 0. */
void mko_resample_wheel(const double* w, int L, int N, double u, const int* fallback, int* idx);
/* Quantise nonnegative weights to integers with 40 bits below the max (exact
 * power-of-two scaling then truncation).  Returns 0 when the reference would
 * take its max-weight-0 fallback (all weights zero/NaN) or a weight is +inf. */
int mko_quantize_f64(const double* w, int L, uint64_t* q);
int mko_quantize_f32(const float* w, int L, uint64_t* q);
/* Exact systematic resampling on integer weights: idx[i] = first j with
 * Q_j >= (i + U/2^32) * Q_{L-1} / N, evaluated in exact 128-bit integers. */
void mko_resample_exact(const uint64_t* q, int L, int N, uint32_t U, int* idx);
/* Full resampler used by every filter: quantise, exact systematic, or the
 * fallback (idx_i = floor(u_i * L), u_i = Philox(key={U, 0x5EED}, ctr={i,0,0,0})).
 * Returns 1 if the fallback was taken. */
int mko_resample_f64(const double* w, int L, int N, uint32_t U, int* idx);
int mko_resample_f32(const float* w, int L, int N, uint32_t U, int* idx);

/* ---- A4/A5: KF_model (KF_model.cpp:11-25), dense reference form */
void mko_kf_predict(int d, const double* F, const double* B, const double* Q, double* x, double* P);
/* mask: bit r set => measurement row r used.  Returns 0 if S is singular. */
int mko_kf_update(int d, int m, const double* H, const double* BH, const double* R,
                  const double* z, unsigned mask, double* x, double* P);

/* ---- A7: Gaussian log density (pf2DRao.cpp:34-67).  mode 0 = exact (intended
 * semantics); 1 = the chol() quirk with OpenCV-2.4 diagonal convention (returned
 * diagonal holds 1/L_ee); 2 = the quirk with the later convention (holds L_ee). */
double mko_mvn_logpdf(int m, const double* x, const double* u, const double* S, int mode);

/* ---- A1: my_gmm::loadGaussian (my_gmm.cpp:45-75), reference form.
 * u: d, s: d*d, Hpca: d*F (pca_proj, rows = PCA dims), mpca: F.  Outputs the
 * component's F,B,Q (d), H (6*d), BH (6), R (6*6). */
void mko_load_gaussian_ref(int d, int Fdim, const double* u, const double* s,
                           const double* Hpca, const double* mpca, double g,
                           double* F, double* B, double* Q, double* H, double* BH, double* R);

/* ---- A1..A10 model + RBPF (pf2DRao.cpp:125-158) */
typedef struct {
  int d, m, K;
  int meas_mode;          /* 0 LINEAR (H x + BH), 1 PINHOLE (EKF per particle) */
  const double* F;        /* K*d*d */
  const double* B;        /* K*d   */
  const double* Q;        /* K*d*d */
  const double* H;        /* K*m*d (LINEAR) */
  const double* BH;       /* K*m   (LINEAR) */
  const double* R;        /* K*m*m */
  const double* weight;   /* K (mixture weights pi) */
  /* PINHOLE: measured joints J = m/2; joint j pixel = pi(Bm_j x + mm_j) */
  const double* Bm;       /* J*3*d */
  const double* mm;       /* J*3   */
  double fx, fy, cx, cy;
} mko_model;

/* Predicted measurement and its Jacobian for state x (LINEAR or PINHOLE). */
void mko_measure(const mko_model* M, int k, const double* x, double* zhat, double* Hx);

/* One ParticleFilter::update (pf2DRao.cpp:125-158) with injected uniforms.
 * x: N*d, P: N*d*d (updated in place, after resampling), z: N*m measurement
 * columns stored row-per-particle, mask: measurement rows used.
 * Outputs (optional, may be NULL): ind (N), logw (N), wn (N normalised), anc (N).
 * alias_prev_anc != NULL (the previous update's ancestors) emulates the shallow
 * cv::Mat copy-assign quirk (pf2DRao.cpp:153-156 with KF_model.cpp:13-24).
 * Returns 1 if the resampling fallback was taken. */
int mko_rbpf_update(const mko_model* M, int N, double* x, double* P, const double* z,
                    unsigned mask, uint32_t U_ind, uint32_t U_anc, const int* alias_prev_anc,
                    int* ind, double* logw, double* wn, int* anc);
/* The same update with the reference's literal pieces, for pinning the oracle
 * against the reference's own update: the resampling wheel (pf2DRao.cpp:175-210)
 * on double uniforms u_ind / u_anc in [0, 1) (fb_ind / fb_anc: the indices of
 * its all-zero branch, or NULL), the Gaussian density in mvn_mode
 * (mko_mvn_logpdf), and weights normalised in the linear domain
 * (pf2DRao.cpp:138-148).  logw_out gets the log density, wn_out the
 * normalised weights. */
int mko_rbpf_update_literal(const mko_model* M, int N, double* x, double* P, const double* z, unsigned mask,
                            double u_ind, const int* fb_ind, double u_anc, const int* fb_anc, int mvn_mode,
                            const int* alias_prev_anc, int* ind_out, double* logw_out, double* wn_out,
                            int* anc_out);
/* getEstimator (pf2DRao.cpp:23-31): uniform mean of track states. */
void mko_rbpf_estimate(int N, int d, const double* x, double* est);

/* ---- A9: PDAF association weights (pfPose.cpp:247-298) over a candidate list.
 * p_a = N(c; hat_a, var I2) (mvnpdf_multiple, pf2DRao.cpp:69-83, 105-122);
 * w_j = L_j / (Pa p_own + Pa p_other + clutter (1 - 2 Pa)); L_j = 1 for detections
 * gives Pa p_own / Z when times Pa (the detection-list adapter).  For a single
 * target (has_other = 0) the denominator is Pa p_own + clutter (1 - Pa). */
void mko_pdaf_weights(int M, const double* cand, const double* Lc, const double* hat_own,
                      const double* hat_other, int has_other, double var, double Pa,
                      double clutter, double* w);

/* ---- A13: bootstrap PF with the mixture motion model (the streaming and batched particle kernels) */
typedef struct {
  int d, K, J;
  const float* a;        /* K*d */
  const float* mb;       /* K*d   (1-a)*mu */
  const float* mu;       /* K*d */
  const float* Lq;       /* K*d(d+1)/2 packed lower, row-major */
  const float* S0c;      /* K*d(d+1)/2 chol(Sigma_k), prior */
  const float* cumpi;    /* K */
  const float* Bm;       /* J*3*d */
  const float* mm;       /* J*3   */
  float fx, fy, cx, cy;
  float kappa, pd, sigma;
} mko_bpf_params;

int mko_pick_component(const float* cumpi, int K, float u);
/* prior draw for one particle: x = mu_k + chol(Sigma_k) eps */
void mko_bpf_prior(const mko_bpf_params* p, const double* eps, float ucomp, double* x);
/* propagate x (d) in place with one particle-frame's draws */
void mko_bpf_propagate(const mko_bpf_params* p, const double* eps, float ucomp, double* x);
/* log-likelihood of the frame's typed detection lists given the state x.
 * det_off: J+1 offsets into det (pairs). */
double mko_bpf_loglik(const mko_bpf_params* p, const double* x, const int* det_off, const float* det);

/* Run whole tracks (timed CPU baseline and end-to-end reference): draws from
 * Philox + libm Box-Muller, resampling with mko_resample_f64 semantics on FP64
 * weights.  Tracks are independent; OpenMP over tracks with nthreads. */
typedef struct {
  int n_particles, n_frames;
  long long frame_base;     /* index of frame 0 in the frame-indexed arrays */
  unsigned long long seed;
  int track_id;
  int param_index;
  float kappa, pd, sigma;
} mko_track;

void mko_bpf_run_tracks(int n_tracks, const mko_track* tracks, int d, int K, int J,
                        const float* a, const float* mb, const float* mu, const float* Lq,
                        const float* S0c, const float* cumpi, const float* Bm, const float* mm,
                        float fx, float fy, float cx, float cy,
                        const int* det_off, const float* det,
                        float* est, float* loglik, float* ess, int nthreads);

/* Teacher-forced FP64 replay of nf consecutive frames of one track (the loop
 * of pf2D.cpp:148-210 with my_gmm.cpp:53-58's motion): each frame starts from
 * this replay's own FP64 particle set, resampled with the ancestors the device
 * chose, propagated with the device's draws, and scored, weighted and averaged
 * in FP64.
 *   x        N*d in/out: the set after the previous frame's propagation (the
 *            prior set before frame 0); on return, the set of the last frame
 *   anc_prev N: the ancestors chosen at the frame before the first (identity
 *            before frame 0)
 *   eps      nf*N*d, ucomp nf*N: the device's draws of the frames
 *   anc      nf*N: the device's ancestors of each frame
 *   w_dev    nf*N: the device's weights (normalised to max 1), or NULL
 *   det_off  nf*J + 1 offsets of the frames' lists into det (pairs)
 * Per frame out: est (nf*d), loglik, ess, and w_err = max_i |w_i - w_dev_i|
 * (w normalised to max 1).  OpenMP over particles. */
void mko_bpf_forced_frames(const mko_bpf_params* p, int N, int nf, double* x, const int* anc_prev,
                           const float* eps, const float* ucomp, const int* anc, const float* w_dev,
                           const int* det_off, const float* det, double* est, double* loglik,
                           double* ess, double* w_err, int nthreads);
/* the prior set of N particles from the device's prior draws (eps N*d, ucomp N) */
void mko_bpf_prior_set(const mko_bpf_params* p, int N, const float* eps, const float* ucomp, double* x,
                       int nthreads);

int mko_num_threads(void);

/* ---- A11: deterministic mixture KF (GPB1 over the K components) with PDAF
 * over each measured joint's candidate list, and its reverse-mode adjoint.
 * Not a single reference function: it is the component-marginalised analogue
 * of ParticleFilter::update (pf2DRao.cpp:125-158, which redraws the component
 * every frame i.i.d. from pi, pf2DRao.cpp:128) built from KF_model
 * (KF_model.cpp:11-25) and the PDA weighting of pfPose.cpp:247-298.
 * Per frame: per component predict (x = a*x + (1-a)*mu, P = A P A + Lq Lq^T),
 * sequential PDAF/EKF updates over the joints (Bar-Shalom combined innovation),
 * l_k = sum_j log[(1-P_D) kappa + P_D sum_i N(z_i; zhat, S)], mixture weights
 * w_k ~ pi_k exp(l_k), c_t = log sum_k pi_k exp(l_k), moment-matched collapse,
 * symmetrisation of P.  logL = sum_t c_t.  Parameters differentiated: mu, a,
 * Lq (packed lower), sigma (R = sigma^2 I2 per joint). */
typedef struct {
  int d, K, J;
  const double* mu;    /* K*d */
  const double* a;     /* K*d */
  const double* Lq;    /* K*d(d+1)/2 */
  const double* pi;    /* K */
  const double* S0;    /* K*d*d prior covariances (not differentiated) */
  double sigma;
  double fx, fy, cx, cy;
} mko_mix_params;

/* one track: T frames at frame_base; Bm (J*3*d), mm (J*3) its body; det_off
 * indexes (global frame g, joint j) lists as for the bootstrap filter */
double mko_mix_forward(const mko_mix_params* p, int T, long long frame_base, const double* Bm,
                       const double* mm, double pd, double kappa, const int* det_off, const float* det);
/* logL and its gradient (accumulated into g_mu (K*d), g_a (K*d), g_Lq (K*DD), g_sigma) */
double mko_mix_adjoint(const mko_mix_params* p, int T, long long frame_base, const double* Bm,
                       const double* mm, double pd, double kappa, const int* det_off, const float* det,
                       double* g_mu, double* g_a, double* g_Lq, double* g_sigma);
/* batch over tracks (OpenMP); body arrays stacked per track; returns sum logL;
 * per-track logL in ll (optional); gradients summed if grad != 0 */
double mko_mix_batch(const mko_mix_params* p, int n_tracks, const int* n_frames, const long long* frame_base,
                     const double* Bm, const double* mm, const double* pd, const double* kappa,
                     const int* det_off, const float* det, int grad, double* ll, double* g_mu,
                     double* g_a, double* g_Lq, double* g_sigma, int nthreads);

/* ---- A12: legacy bootstrap PF pf2D (pf2D.cpp:13-268), literal semantics.
 * my_gmm::loadGaussian (pf2D.cpp:26-37): sigma_i = inv(s), det_s =
 * 1/((2 pi)^(d/2) sqrt(det s)).  update (pf2D.cpp:148-210): prior_i =
 * sum_k w_k det_k expf(float(-1/2 (x-mu_k) S_k^-1 (x-mu_k)^T)), likelihood_i =
 * eyemvnpdf(x[6:8]-z0, 15) * eyemvnpdf(x[0:2]-z1, 15) (pf2D.cpp:124-128),
 * w = prior*lik normalised by their sum; resample (pf2D.cpp:225-268): if the
 * max weight is 0 every column is redrawn uniformly (ctor ranges,
 * pf2D.cpp:44-71; reinit_u: N*d uniforms) and the weights reset to 1/N,
 * otherwise particles <- old[anc] with anc the exact systematic resampling of
 * the normalised weights and the weights left unchanged (the reference never
 * resets them, so getEstimator uses stale weights); predict (pf2D.cpp:90-102):
 * columns 0..7 += N(0, 5^2) (eps: N*8 normals; columns >= 8 get no noise --
 * the reference adds an uninitialised temporary there).
 * particles: N*d, weights: N.  Returns 1 if the re-initialisation ran. */
typedef struct {
  int d, K;
  const double* mean;    /* K*d */
  const double* sinv;    /* K*d*d */
  const double* det_s;   /* K */
  const double* w;       /* K */
  int width, height, side;
} mko_pf2d_model;
void mko_pf2d_load(int d, int K, const double* mean, const double* cov, double* sinv, double* det_s);
void mko_pf2d_init(const mko_pf2d_model* m, int N, const double* u, double* particles, double* weights);
int mko_pf2d_update(const mko_pf2d_model* m, int N, double* particles, double* weights, const double* z,
                    uint32_t U, const double* reinit_u, const double* eps, double* w_out, int* anc_out);
void mko_pf2d_estimate(int N, int d, const double* particles, const double* weights, double* est);

/* ---- f2: pose decode and 3-D back-projection (pfPose.cpp:84-127, 173-208, 347-348)
 * e = Hpca^T x + mpca (F values, Hpca is d x F row-major), then get3Dpose: full
 * state (u, v, Z) for joints hand, elbow, shoulder, head, neck at 0..14, roll,
 * pitch, yaw at 16, 17, 15 and t at 18..20; R = R3(yaw) R2(pitch) R1(roll);
 * P = Kc [R | t]; point k = inv(P[:, 0:3]) ((u Z, v Z, Z) - P[:, 3]) with a
 * 3x3 LU inverse (DECOMP_LU).  pos3d: 3 x 5 row-major (x; y; z rows). */
void mko_pose_decode(int d, int F, const double* Hpca, const double* mpca, const double* x, double* e);
void mko_pose3d(const double* e, const double* Kc, double* pos3d);
/* publish2Dpos record (pfPose.cpp:173-208): 8 (x, y) points: hand1, hand2, head
 * (mean of both arms), neck (mean), elbow1, elbow2, shoulder1, shoulder2 */
void mko_pose2d_record(const double* e1, const double* e2, double* pts16);

/* ---- f1: likelihood-image front end (pfPose.cpp:210-301)
 * GaussianBlur 15x15, sigma 3, BORDER_DEFAULT (reflect-101), as a separable
 * float filter: taps w_k = (float)(exp(-(k-7)^2/18) / sum), each pass the fmaf
 * chain over the taps in order, round to nearest-even, saturate to 8 bits. */
void mko_gaussian_blur_u8(const uint8_t* in, int W, int H, uint8_t* out);
/* candidate likelihoods L = img[(int)y][(int)x] / 255 inside (0 < x < W,
 * 0 < y < H), else 0 (pfPose.cpp:250-254) */
void mko_image_lookup(int M, const double* cand, const uint8_t* img, int W, int H, double* L);

#ifdef __cplusplus
}
#endif
#endif

