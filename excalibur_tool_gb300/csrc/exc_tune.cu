// exc_tune.cu -- launch-schedule autotuner for exc_trace (include/excalibur_gb300.h).
//
// The tracer is latency-bound per photon (dependent gathers and, for FP64, a
// narrow FP64 pipe), so the best (threads per block, resident blocks per SM)
// pair, and whether the a(eta) table is better read from shared memory than
// through the read-only cache (which the grid gathers compete for), depend on
// the precision build, the stepper, the grid sizes and the spread of trajectory
// lengths. This times the real kernel on a caller-given sample for each
// candidate and returns the fastest.
#include <cuda_runtime.h>

#include <cstring>

#include "../../include/excalibur_gb300.h"

namespace exc {
void set_last_error(const char* msg);
}

extern "C" int exc_autotune(const ExcMetric* metric, const ExcTraceArgs* args, const double* pristine_state,
                            ExcLaunchPlan* plan, void* stream) {
  if (!metric || !args || !pristine_state || !plan) {
    exc::set_last_error("autotune: metric, args, pristine_state and plan are required");
    return EXC_ERR_INVALID;
  }
  if (args->dt_state) {
    exc::set_last_error("autotune: args->dt_state must be NULL (trials start from args->dt)");
    return EXC_ERR_INVALID;
  }
  if (args->n_photons < 1 || !args->state) {
    exc::set_last_error("autotune: a non-empty sample is required");
    return EXC_ERR_INVALID;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const size_t bytes = (size_t)args->n_photons * 8 * sizeof(double);
  int cand_b[EXC_TUNE_MAX_TRIALS], cand_p[EXC_TUNE_MAX_TRIALS], n = 0;
  const int per_sm[] = {0, 2, 3, 4, 5, 6, 7, 8};
  for (int b = 32; b <= 128; b += 32)
    for (int p : per_sm)
      if (p * b <= 2048 && n < EXC_TUNE_MAX_TRIALS) {
        cand_b[n] = b;
        cand_p[n] = p;
        ++n;
      }
  const int n_cache = n;
  // the second pass (the staged table) exists for FP64 launches of a metric with a table
  const bool fp64 = args->precision == EXC_PREC_FP64_EXACT || args->precision == EXC_PREC_FP64_FAST ||
                    args->precision == EXC_PREC_MIXED || args->precision == EXC_PREC_RETRACE;
  const bool can_stage = fp64 && metric->kind == EXC_METRIC_FLRW && metric->cosmology != EXC_COSMO_STATIC &&
                         metric->a_table_n <= EXC_STAGING_MAX_TABLE;
  const int n_staged = can_stage ? (EXC_TUNE_MAX_TRIALS - n_cache < 3 ? EXC_TUNE_MAX_TRIALS - n_cache : 3) : 0;
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    exc::set_last_error("autotune: cudaEventCreate failed");
    return EXC_ERR_CUDA;
  }
  memset(plan, 0, sizeof(*plan));
  plan->best_rate = -1.0f;
  int32_t* iters = nullptr;    // host copy of n_iter for the rate
  if (args->n_iter) iters = new int32_t[(size_t)args->n_photons];
  int rc = EXC_SUCCESS;
  int32_t cand_s[EXC_TUNE_MAX_TRIALS] = {0};
  for (int t = -1; t < n_cache + n_staged && rc == EXC_SUCCESS; ++t) {   // t = -1: untimed warm-up
    if (t == n_cache) {
      // second pass: the fastest n_staged schedules of the first, with the staged table
      bool taken[EXC_TUNE_MAX_TRIALS] = {false};
      for (int k = 0; k < n_staged; ++k) {
        int best = -1;
        for (int j = 0; j < n_cache; ++j)
          if (!taken[j] && (best < 0 || plan->trial_rate[j] > plan->trial_rate[best])) best = j;
        taken[best] = true;
        cand_b[n_cache + k] = cand_b[best];
        cand_p[n_cache + k] = cand_p[best];
        cand_s[n_cache + k] = EXC_STAGING_SHARED;
      }
    }
    ExcTraceArgs a = *args;
    a.block_size = t < 0 ? cand_b[0] : cand_b[t];
    a.blocks_per_sm = t < 0 ? cand_p[0] : cand_p[t];
    a.staging = t < 0 ? EXC_STAGING_CACHE : cand_s[t];
    if (cudaMemcpyAsync(a.state, pristine_state, bytes, cudaMemcpyDeviceToDevice, s) != cudaSuccess) {
      exc::set_last_error("autotune: restoring the sample failed");
      rc = EXC_ERR_CUDA;
      break;
    }
    cudaEventRecord(e0, s);
    rc = exc_trace(metric, &a, stream);
    cudaEventRecord(e1, s);
    if (rc != EXC_SUCCESS) break;
    if (cudaEventSynchronize(e1) != cudaSuccess) {
      exc::set_last_error("autotune: trial failed");
      rc = EXC_ERR_CUDA;
      break;
    }
    if (t < 0) continue;
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    double rate = ms > 0.0f ? 1e3 / ms : 0.0;
    if (iters) {
      if (cudaMemcpy(iters, args->n_iter, (size_t)args->n_photons * sizeof(int32_t), cudaMemcpyDeviceToHost) !=
          cudaSuccess) {
        exc::set_last_error("autotune: reading n_iter failed");
        rc = EXC_ERR_CUDA;
        break;
      }
      // photons the launch never reached keep EXC_PH_NOT_RUN and an unwritten n_iter: skip them
      int32_t* st = new int32_t[(size_t)args->n_photons];
      cudaMemcpy(st, args->status, (size_t)args->n_photons * sizeof(int32_t), cudaMemcpyDeviceToHost);
      double sum = 0.0;
      for (int64_t i = 0; i < args->n_photons; ++i)
        if (st[i] != EXC_PH_NOT_RUN) sum += (double)iters[i];
      delete[] st;
      rate = ms > 0.0f ? sum * 1e3 / ms : 0.0;
    }
    plan->trial_block[t] = a.block_size;
    plan->trial_blocks_per_sm[t] = a.blocks_per_sm;
    plan->trial_ms[t] = ms;
    plan->trial_rate[t] = (float)rate;
    plan->trial_staging[t] = a.staging;
    plan->n_trials = t + 1;
    if (rate > plan->best_rate) {
      plan->best_rate = (float)rate;
      plan->best_ms = ms;
      plan->block_size = a.block_size;
      plan->blocks_per_sm = a.blocks_per_sm;
      plan->staging = a.staging;
    }
  }
  delete[] iters;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return rc;
}
