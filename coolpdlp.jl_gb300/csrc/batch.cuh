// batch.cuh -- many independent LPs per call: a persistent kernel with one LP
// per CTA, synchronous (batch_solve) or as an asynchronous job on its own
// stream (submit / poll / cancel / collect) for continuous batching.
#pragma once

#include "cpdlp_common.cuh"

namespace cpdlp {

void batch_solve(Handle& h, int64_t count, const cpdlp_lp* lps, const cpdlp_params* params,
                 double* const* x_out, double* const* y_out, cpdlp_stats* stats);

struct Job;

// Copies the LPs (the caller may free them on return), preprocesses them on
// the job's own stream and launches the solve; returns without waiting for
// it.  reltol (count entries or NULL) gives each LP's target relative KKT
// error; x0 / y0 (count pointers or NULL; NULL entries = cold start) give
// warm starts in original units.  max_ctas > 0 caps the CTAs of each launch
// (leaving SMs to jobs submitted later).
Job* job_submit(Handle& h, int64_t count, const cpdlp_lp* lps, const cpdlp_params* params,
                const double* reltol, const double* const* x0, const double* const* y0,
                int64_t max_ctas);
// true once every LP of the job is finished; takes the LPs finished so far
// and launches the FP64 phase for those that need it.  Never blocks.
bool job_poll(Job* j);
void job_wait(Job* j);
// asks the job's kernels to stop at their next termination check; unfinished
// LPs report CPDLP_STILL_RUNNING
void job_cancel(Job* j);
void job_collect(Job* j, double* const* x_out, double* const* y_out, cpdlp_stats* stats);
// ready[k] = 1 for every LP already finished (its result can be collected)
void job_ready(const Job* j, int32_t* ready);
void job_collect_lp(Job* j, int64_t k, double* x_out, double* y_out, cpdlp_stats* stats);
int64_t job_count(const Job* j);
void job_destroy(Job* j);

// upper bound of the device bytes a job over these LPs holds
int64_t batch_footprint(int64_t count, const cpdlp_lp* lps, const cpdlp_params* params);

}  // namespace cpdlp
