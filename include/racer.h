/* warporacer3d GB300 rollout library: C ABI.
 *
 * Drop-in replacement for the compute beneath the reference's Mojo structs
 * (AlistairKeiller/warporacer3d): Sim (racer/sim.mojo:269-348), Policy and
 * Activations (racer/ppo.mojo:47-138), Trainer (racer/ppo.mojo:141-337),
 * checkpoints (racer/ppo.mojo:341-355) and the benchmark loop's policy step
 * (main.mojo:40-48,82-92). A Mojo host binds these with `external_call`
 * through an `OwnedDLHandle` on libracer.so.
 *
 * Conventions
 *  - Every function returns 0 on success and a nonzero code on failure;
 *    racer_last_error() then describes the failure (per calling thread).
 *    Codes: 1 invalid argument, 2 CUDA error, 3 unsupported.
 *  - Pointers named *_dev are device pointers; buffers are float32 and
 *    feature-major as in the reference: a [rows, n] matrix stores row r at
 *    offset r * n (racer/device.mojo:20-32).
 *  - Each object enqueues its work on the CUDA stream given at creation
 *    (NULL = the legacy default stream) in call order, like the reference's
 *    single DeviceContext queue. Calls on one object are not re-entrant;
 *    distinct objects may be used from distinct threads.
 *  - Functions that return host values (racer_trainer_rollout's mean reward,
 *    racer_trainer_update's KL, racer_download) synchronise the stream, as
 *    the reference's device.read does.
 */
#ifndef RACER_H
#define RACER_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RACER_STATE 11 /* state rows: x y z heading speed steer steps progress episode friction return */

/* ---- errors and memory helpers (racer/device.mojo:48-54,121-134) ---- */
const char* racer_last_error(void);
int racer_version(void);
int racer_alloc(size_t bytes, void** dev);                                   /* device.alloc, zero-filled */
int racer_free(void* dev);
int racer_upload(void* dev, const void* host, size_t bytes, void* stream);   /* device.write */
int racer_download(void* host, const void* dev, size_t bytes, void* stream); /* device.read */
int racer_synchronize(void* stream);

/* ---- Sim: racer/sim.mojo:269-348 ---- */
typedef struct racer_sim racer_sim;
typedef struct {
  float* state;       /* [11, n] */
  float* obs;         /* [beams + 5, n]; row beams + 4 is the constant 1 */
  float* actions;     /* [2, n] steer, throttle in [-1, 1] */
  float* reward;      /* [n] */
  float* done;        /* [n] 0 running, 1 crash, 2 timeout */
  const float* track; /* the track array, uploaded unchanged */
} racer_sim_buffers;

/* Sim.__init__ (racer/sim.mojo:280-289): uploads the track array
 * (racer/track.py:15-18 layout) and allocates n cars. beams >= 2. */
int racer_sim_create(const float* track, size_t len, int n, uint64_t seed, int beams, void* stream,
                     racer_sim** out);
/* Several tracks in one sim (no counterpart in the reference, where a Sim
 * holds one Map): `count` (1..8) segments, segment k = cars[k] cars on
 * tracks[k] (lens[k] floats) seeded by seeds[k]. The buffers are [rows,
 * sum(cars)] with segment k in columns [cars[0] + ... + cars[k-1], ...).
 * Each kernel launch covers every segment, and segment k evolves exactly as
 * racer_sim_create(tracks[k], lens[k], cars[k], seeds[k], ...) would (its
 * cars' Philox counters are their indices within the segment); policy sampling
 * uses seeds[0] over the whole batch. racer_sim_create is the one-segment case. */
int racer_sim_create_segments(int count, const float* const* tracks, const size_t* lens, const int* cars,
                              const uint64_t* seeds, int beams, void* stream, racer_sim** out);
/* Lidar launch shape (no counterpart in the reference). cars_per_block: cars
 * (warps) per block, 2, 4 or 8. wide: 1 selects the kernel compiled for 48
 * resident warps per SM (40 registers a thread) instead of 64 (32 registers).
 * split (several segments only): 0 = one launch covering every segment
 * through the segment table; 1 = each segment's one-track kernel on its own
 * stream, forked from and joined into the sim's stream (parallel branches of
 * a captured rollout graph). order[0..count): the segments' order in the grid
 * (split = 0) or their launch order (split = 1). dynamic (one-track sims and
 * split launches): 1 = a persistent grid per segment whose warps take (car,
 * 32-beam group) units from an atomic counter instead of a fixed block per
 * group of cars (cars_per_block is then unused). flat (one-track sims and
 * split launches, not dynamic): 1 = each warp takes the next 32 (car, beam)
 * pairs in car-major order, across car boundaries, so no lane idles when the
 * beam count is not a multiple of 32. Setting a different shape drops the
 * sim's captured rollout graphs. */
typedef struct {
  int cars_per_block;
  int wide;
  int split;
  int dynamic;
  int order[8];
  int flat;
} racer_lidar_shape;
int racer_sim_set_lidar_shape(racer_sim* sim, const racer_lidar_shape* shape);
int racer_sim_get_lidar_shape(racer_sim* sim, racer_lidar_shape* shape);
/* Autotuner: times `reps` lidar passes on the sim's current lidar frames for
 * every cars_per_block, wide, dynamic, flat and (with several segments)
 * split, with the segments in index order and heaviest-first (by probe
 * iterations counted in one pass), in two rounds over all shapes; keeps the
 * shape with the fastest round and returns it with that round's mean time in
 * ms. The lidar only rewrites obs rows from the frames: the sim's state is
 * unchanged. */
int racer_sim_autotune(racer_sim* sim, int reps, racer_lidar_shape* best, float* best_ms);
/* Rollout graphs (racer_rollout) as `chains` (1..16) independent chains of
 * Runner steps over consecutive car ranges (multiples of 128), forked from and
 * joined into the sim's stream, so one chain's policy forward and physics run
 * beside another chain's lidar. Cars never interact, so every result is the
 * one-chain rollout's. Applies to one-track sims with a BF16 policy; drops
 * captured graphs. */
int racer_sim_set_chains(racer_sim* sim, int chains);
/* Rollout graphs (racer_rollout) as one launch of the fused persistent kernel
 * (enable = 1; one-track sims with a BF16 policy, else ignored): each CTA owns
 * a slice of at most 128 cars for all steps and runs, step after step, the
 * policy forward on the tensor cores with the sampling, the physics and the
 * lidar of its cars, the observations never leaving the SM's L2 slice between
 * phases. Every result is the chained graph's (racer/sim.mojo:307-321,
 * main.mojo:40-48 per step). 0 (the default) = kernels per step. Drops
 * captured graphs. */
int racer_sim_set_fused_rollout(racer_sim* sim, int enable);
int racer_sim_destroy(racer_sim* sim);
int racer_sim_get_buffers(racer_sim* sim, racer_sim_buffers* out);
/* Sim.reset (racer/sim.mojo:291-305): spawn every car, then a step at rest. */
int racer_sim_reset(racer_sim* sim);
/* Sim.step (racer/sim.mojo:307-321): physics for every car, then the lidar.
 * actions [2, n], reward [n], done [n], obs [beams + 5, n] are device views
 * (for example slices of rollout storage). */
int racer_sim_step(racer_sim* sim, const float* actions_dev, float* reward_dev, float* done_dev, float* obs_dev);
/* Sim.step that also records the probe iterations of every beam into
 * iters_dev [beams, n] (int32): the measured per-beam work. */
int racer_sim_step_counted(racer_sim* sim, const float* actions_dev, float* reward_dev, float* done_dev,
                           float* obs_dev, int32_t* iters_dev);
/* Sim.sample (racer/sim.mojo:323-348): output [3, n], log_std [2] ->
 * actions [2, n], logp [n], value [n]. */
int racer_sim_sample(racer_sim* sim, const float* output_dev, const float* log_std_dev, float* actions_dev,
                     float* logp_dev, float* value_dev, int deterministic, int64_t step);

/* ---- Policy and Activations: racer/ppo.mojo:47-138 ---- */
typedef struct racer_policy racer_policy;
typedef struct racer_acts racer_acts;
/* Policy.__init__ (racer/ppo.mojo:68-90) for IN = beams + 5 inputs. */
int racer_policy_create(int beams, uint64_t seed, void* stream, racer_policy** out);
int racer_policy_destroy(racer_policy* policy);
/* theta [P] = W0 [64, IN] | W1 [64, 65] | W2 [3, 65] | log std [2]. */
int racer_policy_theta(racer_policy* policy, float** theta_dev, int* p);
/* Call after writing theta directly (a checkpoint load): refreshes the
 * policy's derived weight copies. */
int racer_policy_sync(racer_policy* policy);
/* Precision of the forward, backward and weight-gradient products: 1 (the
 * default) = BF16 operands on the tcgen05 tensor cores with FP32
 * accumulation; 0 = FP32 on the CUDA cores (the same-seed comparison run).
 * Parameters, sampling and Adam stay FP32 either way. */
int racer_policy_set_precision(racer_policy* policy, int bf16);
/* Activations.__init__ (racer/ppo.mojo:56-60): h1, h2 [65, cols] with row 64 = 1, o [3, cols]. */
int racer_acts_create(racer_policy* policy, int cols, racer_acts** out);
int racer_acts_destroy(racer_acts* acts);
int racer_acts_buffers(racer_acts* acts, float** h1_dev, float** h2_dev, float** o_dev);
/* Policy.forward (racer/ppo.mojo:108-111): x [IN, cols]. */
int racer_policy_forward(racer_policy* policy, const float* x_dev, racer_acts* acts);
/* Policy.backward (racer/ppo.mojo:113-138): d3 [3, cols] -> d2, d1 [65, cols],
 * W0/W1/W2 entries of grad [P]. */
int racer_policy_backward(racer_policy* policy, const float* x_dev, racer_acts* acts, const float* d3_dev,
                          float* d2_dev, float* d1_dev, float* grad_dev);
/* Policy.backward for callers that cannot allocate device memory (their
 * device memory belongs to another runtime's allocator, such as a Mojo/MAX
 * DeviceContext, or to a fixed up-front budget). It has no counterpart in the
 * reference. Every buffer is the caller's: theta [P] for IN = beams + 5,
 * x [IN, cols], h1/h2 [65, cols] from a forward, d3 [3, cols]; it writes
 * d2, d1 [65, cols] and the W0/W1/W2 entries of grad [P], the same values as
 * racer_policy_backward in FP32 precision (its CUDA-core split-K products).
 * The split-K scratch is a 4.75 MiB array inside the
 * library (one per GPU, held until exit); no call allocates or frees. The
 * first call on a device resolves the array's address (make it before any
 * stream capture) and keeps it, so do not use it on a device after a
 * cudaDeviceReset; calls that overlap on the GPU race on the array. */
int racer_policy_backward_noalloc(int beams, const float* theta_dev, const float* x_dev, int cols,
                                  const float* h1_dev, const float* h2_dev, const float* d3_dev, float* d2_dev,
                                  float* d1_dev, float* grad_dev, void* stream);
/* Error word of the policy's tensor-core kernels (0 = none; nonzero when a
 * bounded wait on the tensor core timed out), read and cleared. A kernel whose
 * wait timed out issues no further copy or MMA, lets those it issued complete,
 * frees its tensor memory and returns; its outputs are then undefined.
 * Synchronises the policy's stream. */
int racer_policy_status(racer_policy* policy, int* code);
/* Test of the timeout mechanism (no counterpart in the reference): launches,
 * on the policy's stream, a one-CTA tensor-core kernel that holds tensor
 * memory and waits on an mbarrier nothing will ever arrive on, issuing no
 * copy, MMA or tensor-memory load. Its bounded wait gives up after `polls`
 * (>= 1) polls, it records the timeout in the policy's error word (read by
 * racer_policy_status), frees its tensor memory and returns. */
int racer_policy_wait_test(racer_policy* policy, int polls);
/* save/load (racer/ppo.mojo:341-355): one float32 .npy holding [iteration, theta]. */
int racer_policy_save(racer_policy* policy, const char* path, int iteration);
int racer_policy_load(racer_policy* policy, const char* path, int* iteration);

/* ---- Trainer: racer/ppo.mojo:141-337 (rollout length is a parameter) ---- */
typedef struct racer_trainer racer_trainer;
typedef struct racer_surrogate racer_surrogate; /* the learned lidar, declared with its functions below */
typedef struct {
  float *obs, *actions, *logp, *value, *reward, *done, *advantage; /* rollout storage */
  float *x, *d3, *d2, *d1, *grad, *first, *second, *stats;         /* minibatch scratch (x: [4][IN, batch], the
                                                                      four minibatches' inputs), Adam, stats[5] */
  racer_acts* acts;                                                  /* the minibatch activations */
  int batch;
} racer_trainer_buffers;
int racer_trainer_create(int n, int beams, int rollout, void* stream, racer_trainer** out);
int racer_trainer_destroy(racer_trainer* trainer);
int racer_trainer_get_buffers(racer_trainer* trainer, racer_trainer_buffers* out);
/* Trainer.rollout (racer/ppo.mojo:187-232): returns the mean reward per step. */
int racer_trainer_rollout(racer_trainer* trainer, racer_sim* sim, racer_policy* policy, racer_acts* acts,
                          int iteration, float* mean_reward);
/* Rollouts of racer_trainer_rollout with the learned lidar (no counterpart in
 * the reference, whose Trainer.rollout traces every step, racer/ppo.mojo:187-232):
 * after each physics step the lidar rows of the rollout storage come from
 * `surrogate` (bound to the rollout's sim), every `audit_every`-th step of
 * training (iteration * rollout + t, 0 = never) is traced exactly for all cars
 * and its error accumulated (racer_surrogate_rollout_stats), and on the other
 * steps each car whose smallest predicted range is below `fallback_m` metres is
 * traced exactly. surrogate = NULL restores exact tracing. */
int racer_trainer_set_surrogate(racer_trainer* trainer, racer_surrogate* surrogate, int audit_every, float fallback_m);
/* Trainer.update (racer/ppo.mojo:234-257): returns the last minibatch's KL estimate. */
int racer_trainer_update(racer_trainer* trainer, racer_policy* policy, float* kl);
/* Updates replay one captured CUDA graph per policy (taken on the update after
 * the first of a policy's configuration; the same launches and results as the
 * eager update). enable = 0 runs every update eagerly. */
int racer_trainer_set_graphs(racer_trainer* trainer, int enable);
/* Trainer.minibatch (racer/ppo.mojo:259-315) with explicit advantage moments. */
int racer_trainer_minibatch(racer_trainer* trainer, racer_policy* policy, int m, float adv_mean, float adv_scale);

/* ---- Runner policy step (main.mojo:40-48) and graph-captured rollouts ---- */
/* One step of every car acting with the policy: forward on sim obs, sample
 * into sim actions (logp and value into scratch_dev [2, n]), Sim.step. */
int racer_runner_step(racer_sim* sim, racer_policy* policy, racer_acts* acts, float* scratch_dev,
                      int deterministic, int64_t t);
/* `steps` consecutive Runner steps replayed from one CUDA graph (captured on
 * first use for each (policy, acts, steps, deterministic)); the sampling
 * offsets are step0, step0 + 1, ... */
int racer_rollout(racer_sim* sim, racer_policy* policy, racer_acts* acts, float* scratch_dev, int steps,
                  int deterministic, int64_t step0);
/* Autotuner for the rollout graph: times `reps` rollouts of `steps` stochastic
 * Runner steps for 1, 2, 3, 4, 6, 8, 12 and 16 chains and (one-track sims, BF16 policy) the fused
 * persistent kernel (after one warm-up rollout each; the sim state advances),
 * keeps the fastest and returns it with its env-steps/s; best_chains = 0
 * means the fused kernel won. */
int racer_runner_tune_chains(racer_sim* sim, racer_policy* policy, racer_acts* acts, float* scratch_dev, int steps,
                             int reps, int* best_chains, float* best_rate);
/* Runner.evaluate (main.mojo:70-80): `steps` deterministic Runner steps
 * (sampling offsets step0, step0 + 1, ...) replayed from one CUDA graph in
 * which the physics kernel adds every car's reward (FP64) and crash to
 * per-car sums on the device; one fixed-order reduction and one read at the
 * end replace the reference's two blocking reads per step. out[0] = reward
 * per car-step, out[1] = crashes per car. */
int racer_runner_evaluate(racer_sim* sim, racer_policy* policy, racer_acts* acts, float* scratch_dev, int steps,
                          int64_t step0, double* out);
/* Serve snapshot (main.mojo:94-124, without the HTTP bridge and viewer):
 * state, obs, actions, reward and done of every car, in that order,
 * (11 + beams + 5 + 4) * n floats, packed on the device and copied to `host`
 * by one asynchronous copy on the sim's stream (use pinned memory for an
 * asynchronous copy); synchronize != 0 waits for it. */
int racer_sim_snapshot(racer_sim* sim, float* host, int synchronize);
/* Accuracy audit of the binary32 dynamics (no counterpart in the reference):
 * `steps` Runner steps as racer_runner_step, and after each one a kernel
 * re-integrates racer/sim.mojo:189-213 in FP64 from the pre-step state and
 * the same actions for every car that did not end its episode. out[7] (host):
 * cars audited, then the sums and then the maxima of the position (m),
 * heading (rad) and speed (m/s) differences. */
int racer_runner_audit_dynamics(racer_sim* sim, racer_policy* policy, racer_acts* acts, float* scratch_dev,
                                int deterministic, int steps, int64_t step0, double* out);

/* ---- learned lidar surrogate (no counterpart in the reference; replaces
 * racer/sim.mojo:238-266's tracing during rollouts, audited by it) ---- */
/* MLP from the lidar frame (origin x, y, z; sin/cos heading; layer one-hot;
 * constant 1; fixed Fourier features of x, y, z and heading: 64 inputs)
 * through three tanh layers of `hidden` (128, 256 or 512) to the sim's
 * `beams` ranges / 10 m, for the sim's track (at most two layers).
 * `batch` (a multiple of 128) is the training batch; `seed` the init. */
int racer_surrogate_create(racer_sim* sim, int hidden, int batch, uint64_t seed, racer_surrogate** out);
/* frame 0: as racer_surrogate_create (one output per beam, the car frame).
 * frame 1: the world frame: the network predicts the range profile at
 * K = 4 (beams - 1) / 3 fixed world angles (the beam spacing; beams - 1 must
 * be a multiple of 12) and beam b of a car reads the sample at its heading's
 * offset plus b, so the rotation by the heading is exact rather than learned;
 * the inputs are trainable feature grids per layer at the origin (five
 * resolutions, eight features each), fixed Fourier features of x and y and
 * the sub-sample phase of the heading.
 * frame 2: the car frame's outputs (one per beam) from the same feature grids
 * beside the frame, heading harmonics and two Fourier octaves. */
int racer_surrogate_create_frame(racer_sim* sim, int hidden, int batch, uint64_t seed, int frame,
                                 racer_surrogate** out);
int racer_surrogate_destroy(racer_surrogate* surrogate);
/* FP32 master parameters W1 [H,64] | W2 [H,H] | b2 [H] | W3 [H,H] | b3 [H] |
 * W4 [nout,H] | b4 [nout] (nout = beams, or K in the world frame) | (world
 * frame and frame 2, from the next multiple of 8) the feature grids, level by level
 * [layers][gy][gx][8], and their last gradient (device pointers). */
int racer_surrogate_params(racer_surrogate* surrogate, float** theta_dev, float** grad_dev, long* count, int* hidden);
/* The feature-grid geometry (frames 1 and 2): per level (5) the vertex
 * counts gx, gy, the spacing in metres and the offset of the level's block in
 * the parameters (null pointers are skipped); fails without feature grids. */
int racer_surrogate_grid(racer_surrogate* surrogate, int* gx, int* gy, float* spacing_m, long* offset);
/* The encoded inputs (host, [batch, 64], the BF16 values as float) and, in the
 * world frame, each sample's first world sample k0 (host, [batch]) of the
 * batch of the last racer_surrogate_gradient call. */
int racer_surrogate_batch_inputs(racer_surrogate* surrogate, float* inputs, int* k0);
/* The surrogate's predictions (ranges / 10 m, clamped to [0, 1]) for that
 * batch into pred_dev [beams, batch], through the rollouts' layered inference
 * path (in the world frame: FP16 profiles, then the gather by heading). */
int racer_surrogate_batch_predict(racer_surrogate* surrogate, float* pred_dev);
/* Training set: `count` poses (a multiple of the batch), uniform over the
 * drivable cells of every layer, heading uniform in (-pi, pi). */
int racer_surrogate_set_poses(racer_surrogate* surrogate, long count, uint64_t seed);
/* Device pointer to the pose set: float4 (x, y, heading, layer) per pose. */
int racer_surrogate_poses(racer_surrogate* surrogate, void** poses_dev, long* count);
/* Gradient of the mean squared range error (ranges / 10 m) of the batch of
 * poses starting at `first`, labelled by the exact tracer; no update.
 * label_dev_out (optional) gets the labels [beams, batch]. */
int racer_surrogate_gradient(racer_surrogate* surrogate, long first, float* mse, float* label_dev_out);
/* `steps` Adam steps over consecutive batches (cosine decay from lr to lr/100);
 * returns the last batch's mean squared error and mean absolute error in metres. */
int racer_surrogate_train(racer_surrogate* surrogate, int steps, float lr, float* last_mse, float* last_mae_m);
/* Training loss: huber_m = 0 (the default) is the squared range error; > 0 the
 * Huber loss with that threshold in metres (gradient clamped beyond it). */
int racer_surrogate_set_loss(racer_surrogate* surrogate, float huber_m);
/* Use the surrogate with another sim on the same track array (same header,
 * length and beam count), for example a trained surrogate driving training
 * runs of several seeds; drops the old sim's learned-lidar rollout graphs. */
int racer_surrogate_bind(racer_surrogate* surrogate, racer_sim* sim);
/* Rollout inference of a 512-wide surrogate: 1 (the default) = one fused
 * kernel (all four layers per tile of 128 cars, activations kept on chip);
 * 0 = four GEMM launches. Both give the same bits. Drops captured rollout graphs. */
int racer_surrogate_set_fused(racer_surrogate* surrogate, int fused);
/* Keep the training set's exact labels after their first tracing (enable = 1,
 * the default; FP32, built by racer_surrogate_set_poses when the set's labels
 * fit in 32 GB) so later epochs copy instead of tracing again: the same bits.
 * enable = 0 traces every batch every time (and frees the cache). */
int racer_surrogate_set_label_cache(racer_surrogate* surrogate, int enable);
/* Held-out error on `batches` fresh batches drawn with `seed`, surrogate vs exact. */
int racer_surrogate_evaluate(racer_surrogate* surrogate, int batches, uint64_t seed, float* mae_m, float* rmse_m,
                             float* max_m, float* frac_over_5cm);

/* Spot check between audits (no counterpart in the reference; off, stride 0,
 * by default): on every non-audit step of a learned-lidar rollout, beams
 * (step % stride) + k * stride of every car are traced exactly and compared
 * with the prediction; a car with one off by more than tolerance_m metres
 * (too long, a missed wall, as well as too short) falls back to the exact
 * tracer for all its beams, like a car under the fallback threshold. */
int racer_surrogate_set_spot_check(racer_surrogate* surrogate, int stride, float tolerance_m);
/* `steps` Runner steps from one CUDA graph with the lidar rows of the
 * observations predicted by `surrogate` (built for this sim): every
 * `audit_every`-th step (0 = never) is traced exactly for all cars and the
 * prediction error accumulated; on the other steps each car whose smallest
 * predicted range is below `fallback_m` metres is traced exactly. */
int racer_rollout_surrogate(racer_sim* sim, racer_policy* policy, racer_acts* acts, float* scratch_dev,
                            racer_surrogate* surrogate, int steps, int deterministic, int64_t step0, int audit_every,
                            float fallback_m);
/* Audited error (metres) and the fraction of non-audit car-steps that fell
 * back to the exact tracer, since the last reset (reset != 0 clears them). */
int racer_surrogate_rollout_stats(racer_surrogate* surrogate, float* mae_m, float* rmse_m, float* max_m,
                                  float* frac_over_5cm, float* fallback_frac, int reset);

/* ---- dense products (Device.gemm with transpose_b, racer/device.mojo:82-98) ---- */
/* C[M, N] (float32, row-major, ldc) = A[M, K] . B[N, K]^T on the tcgen05 tensor
 * cores with BF16 operands (row-major, K contiguous, lda/ldb multiples of 8,
 * 16-byte aligned) and FP32 accumulation. splits > 1 divides K across CTAs and
 * needs scratch_dev of splits * M * N floats. err_dev (int, device) is set
 * nonzero if a bounded wait inside the kernel timed out. */
int racer_gemm_bf16(const void* a_dev, const void* b_dev, float* c_dev, int M, int N, int K, int lda, int ldb,
                    int ldc, int splits, float* scratch_dev, int* err_dev, void* stream);

/* ---- track compilation (racer/track.py:54-125) ---- */
/* One ramp box (racer/track.py:111-116): centre, cos and sin of its heading,
 * length, width, height and rise (the reference's default rise is length / 2). */
typedef struct racer_ramp {
  double cx, cy, cos_heading, sin_heading, length, width, height, rise;
} racer_ramp;
/* The grids of a ribbon track on the GPU: the per-cell loop of
 * racer/track.py:73-104 (`ribbon`) and the fill and blur of :108-121 (`pack`).
 * route [W][3] is the resampled route (racer/track.py:66), cos_h / sin_h the
 * cos and sin of its headings and grade its z gradient (:67-68), computed as
 * the reference computes them; x0, y0, nx, ny the grid of :69-71. Writes
 * grids [layers][3][ny * nx] (clearance, height, waypoint; grids_len >= 6 * nx *
 * ny) and *layers (1 or 2): the floats between the packed array's header and
 * route (:122-125), equal to the reference's. Returns 4 if a cell lies under
 * more than 8 passes of the route, 3 if no cell lies on the road. */
int racer_track_ribbon(const double* route, const double* cos_h, const double* sin_h, const double* grade,
                       int waypoints, double half_width, double bank, double x0, double y0, double cell, int nx,
                       int ny, const double* ramps, int n_ramps, float* grids, int64_t grids_len, int* layers);
/* The grids of an occupancy-image track on the GPU (racer/track.py:56-58 and
 * pack :108-121): free [ny * nx] (nonzero = drivable, rows south to north),
 * route [W][3] the resampled centreline (:54-55). Writes grids [3][ny * nx].
 * Returns 3 unless the image has both free and occupied cells. */
int racer_track_image(const uint8_t* free_cells, const double* route, int waypoints, double x0, double y0,
                      double cell, int nx, int ny, const double* ramps, int n_ramps, float* grids,
                      int64_t grids_len);

/* ---- measurement ---- */
/* Kernel launches in the CUDA graph racer_rollout replays for these arguments
 * (captured here if needed), plus the one launch that sets its step offset. */
int racer_rollout_kernel_count(racer_sim* sim, racer_policy* policy, racer_acts* acts, float* scratch_dev, int steps,
                               int deterministic, int64_t* count);
/* Times `reps` launches of the physics kernel and of the lidar kernel on the
 * sim's stream with CUDA events (actions as given; the sim state advances),
 * returning their mean durations in ms and the probe iterations of the last
 * lidar pass summed over all beams. */
int racer_sim_profile(racer_sim* sim, const float* actions_dev, int reps, float* physics_ms, float* lidar_ms,
                      int64_t* probe_iterations);
/* The roofline of random gathers from L2 (no counterpart in the reference):
 * times `reps` launches in which every thread of 8 CTAs per SM makes random,
 * independent 16-byte loads (8 in flight) from a zeroed buffer of `bytes` (a
 * power of two, 4 KB to 256 MB; L2-resident when it fits the L2), as the
 * lidar gathers its cells, and returns the bytes loaded per second in GB/s. */
int racer_gather_peak(size_t bytes, int reps, float* gbs);

#ifdef __cplusplus
}
#endif
#endif /* RACER_H */
