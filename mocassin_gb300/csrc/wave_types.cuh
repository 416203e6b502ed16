// wave_types.cuh -- host/device parameter blocks of the chosen (wavefront)
// form.  All arrays are device memory owned by the context.
#pragma once

#include <cuda_runtime.h>

#include "mc_device.cuh"

namespace mcg {

// Round entry counts passed as this value are read from the device (the
// previous march's a_count) instead: the form whose rounds run inside one
// CUDA graph.
constexpr unsigned int kDeviceCount = 0xFFFFFFFFu;

// a cell's (x, y, z) in one word, 10 bits each (the device's pack_cell)
__host__ __device__ inline uint32_t pack_cell_host(int x, int y, int z) {
  return (uint32_t)x | ((uint32_t)y << 10) | ((uint32_t)z << 20);
}

struct WaveGrid {
  // march-indexed views of the grid
  const float *opac;        // [nb][S] opacity
  const float *sca;         // [nb][S] dust scattering opacity, or null
  double *jste;             // [nb][S]
  double *jdif;             // [nb][S] or null
  long long S;              // slab stride
  int off;                  // ci = lin + off
  int identity;             // active(lin) == lin + 1 for every cell
  const int32_t *lin2cell;  // [nx*ny*nz] active value at lin
  int refill_min;           // free lanes that trigger a warp's refill
  int inner_steps;          // crossings per lane between refills (fast path)
  // per-round sampling (indexed by packet id in round 0, by absorbed-list
  // index in later rounds)
  uint16_t *s_nu;           // sampled bin, 0xFFFF = no march
  uint32_t *s_words;        // draws consumed after the sampling
  // frequency sort
  unsigned int *bin_count;  // [nb]; bin_count[0] = queue length after the scan
  unsigned int *bin_cursor; // [nb]
  unsigned long long *qhead;
  uint32_t *queue;          // [qlen] sort order (ids or absorbed indices)
  // queue entries in sorted order, written by the emission pass
  uint32_t *q_id, *q_cell, *q_words, *q_meta;
  int32_t *q_origin;
  void *q_r, *q_v, *q_pass; // Real[3], Real[3], Real
  // packets absorbed in this round (the next round's input)
  unsigned int *a_count;
  unsigned int *n_round;    // the round's entry count, kept before the scan resets a_count (graph form)
  int *round_ctr;           // rounds run so far (graph form)
  uint32_t *a_id, *a_cell, *a_words;
  uint16_t *a_run;
  void *a_r;                // Real[3]
};

// One model of a batched march (wave_march_batch_kernel).
struct BatchModel {
  DevGrid g;
  DevSources S;
  WaveGrid w;
  DevCounters *cnt;
  unsigned int task_end;  // tasks of models 0..this one in one pass
};

struct BatchLaunch {
  const BatchModel *models;   // device array
  int nmodels;
  unsigned int tasks_per_pass;
  unsigned int *task_ctr;     // device, zeroed before the launch
  size_t smem;                // dynamic shared memory: the largest model's
  int blocks;                 // from launch_wave_march_batch_blocks_*
  bool dust;
  cudaStream_t stream;
};

struct WaveLaunch {
  DevGrid g;
  DevSources S;
  DevReplay rp;
  WaveGrid w;
  DevCounters *cnt;
  int num_sms;
  cudaStream_t stream;
};

}  // namespace mcg
