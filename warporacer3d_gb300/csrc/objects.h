// Internal definitions of the C-ABI objects shared by the library's host
// translation units (api.cu, surrogate.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <map>
#include <vector>
#include <tuple>

#include "../../include/racer.h"
#include "common.cuh"

// Sim (racer/sim.mojo:269-289): cars on one or more tracks (a segment table,
// one car range per track) and their buffers on one stream.
struct racer_sim {
  int n = 0, beams = 0, in_rows = 0;
  uint64_t seed = 0;  // sampling seed (the first segment's)
  size_t track_len = 0;
  racer::TrackDev t{};  // the first segment's track
  racer::Segments seg{};
  racer::LidarShape shape{};
  float* d_track = nullptr;  // the first segment's uploads (also in seg_track / seg_cl)
  float2* d_cl = nullptr;
  std::vector<float*> seg_track;
  std::vector<float2*> seg_cl;
  // per-segment lidar launches (LidarShape::split): streams and events of the fork/join
  std::vector<cudaStream_t> aux;
  std::vector<cudaEvent_t> join;
  cudaEvent_t fork = nullptr;
  unsigned* counters = nullptr;  // [MAX_SEGMENTS] unit counters of the dynamic lidar
  // rollouts as independent chains over car ranges (parallel branches of the graph)
  int chains = 1;
  // 1: rollout graphs are one launch of the fused persistent kernel (racer_sim_set_fused_rollout)
  int fused = 0;
  std::vector<cudaStream_t> chain_st;
  std::vector<cudaEvent_t> chain_join;
  cudaEvent_t chain_fork = nullptr;
  // device-side evaluation: per-car reward (FP64) and crash sums, and the two totals
  double* eval_reward = nullptr;
  int* eval_crash = nullptr;
  double* eval_total = nullptr;
  std::map<std::tuple<const void*, const void*, const void*, int>, cudaGraphExec_t> eval_graphs;
  float* snapshot = nullptr;  // [(STATE + IN + 4) * n] staging for one-copy snapshots
  int sms = 152;
  float2* beam_dir = nullptr;
  float4* ray = nullptr;  // [2, n] per-car lidar frame written by the physics kernel
  float *state = nullptr, *obs = nullptr, *actions = nullptr, *reward = nullptr, *done = nullptr;
  int64_t* step_base = nullptr;
  cudaStream_t st = nullptr;
  bool owned = false;
  std::map<std::tuple<const void*, const void*, const void*, int, int>, cudaGraphExec_t> graphs;
  std::map<std::tuple<const void*, const void*, const void*, int, int>, size_t> graph_kernels;
  // rollouts with the learned lidar: (policy, acts, scratch, steps, det, surrogate, audit_every, fallback)
  std::map<std::tuple<const void*, const void*, const void*, int, int, const void*, int, float>, cudaGraphExec_t>
      surrogate_graphs;
};
