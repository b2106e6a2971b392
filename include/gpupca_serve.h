/*
 * gpupca_serve.h — projection serving on a resident reference panel (no counterpart API in
 * the reference: smartpca projects non-PCA samples with lsqproj, src/eigensrc/smartpca.c
 * :4606-4757, one run per sample set; here the panel stays in HBM and requests stream in).
 *
 * A server is opened from a handle after gp_snp_weights: it copies the panel (the kept SNPs,
 * their xmean/xfancy, E = fxscal_j ffvecs_js and the K(K+1)/2 pair products of E) into its
 * own device memory, cuts the panels into fp16 slices once, and starts a scheduler thread.
 *
 * Requests carry nsamp new samples as 2-bit codes, one row of row_bytes bytes per sample over
 * the panel's SNPs in panel order (byte s>>2, bits (3-(s&3))*2, MSB first, 3 = missing; pad
 * codes 3).  A request is admitted as soon as it fits in the device pool (pool_samples rows,
 * a FIFO ring): admission starts its host->device copy on a copy stream.  The scheduler packs
 * every admitted request into the next batch (up to max_batch samples), runs the masked
 * normal equations as exact tensor-core products plus the per-sample FP64 Cholesky solves,
 * keeps two batches in flight, and completes requests in order.  Requests that arrive while
 * a batch runs join the next one (continuous batching); their copies overlap the running
 * batch.  Products are exact integer sums, so a sample's coordinates do not depend on which
 * other requests share its batch.
 *
 * The batches run in one persistent launch: a CUDA graph whose while-loop body takes the next
 * batch from a request queue in mapped host memory (a device kernel waits, bounded by a poll
 * interval, for published requests and packs every contiguous one up to max_batch rows), runs
 * the two tensor-core products and the solves on that batch's rows, writes the coordinates
 * and statuses into mapped host memory at the requests' pool rows and publishes the count of
 * completed requests.  The host thread only copies request rows in, publishes them, and
 * hands results back; the loop ends when the server closes.  host_loop = 1 keeps the
 * previous schedule (one set of launches per batch from the host thread).
 *
 * Full-PCA jobs (gp_serve_submit_pca) share the server: they are admitted by estimated device
 * footprint and run on worker handles beside the projection batches.
 *
 * Outputs per sample: coords [nsamp*K] (sample q, eigenvector j at q*K + j), scaled by the
 * opts' eigscale; status 0 ok, 1 = at most K observed SNPs (dropped, coords 0), 2 = normal
 * equations not positive definite (coords 0).  The caller's code buffer must stay valid and
 * the output buffers untouched until the request completes.
 */
#ifndef GPUPCA_SERVE_H
#define GPUPCA_SERVE_H

#include <stdint.h>

#include "gpupca.h"
#include "gpupca_run.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gp_server gp_server;

typedef struct {
  int32_t numeigs;       /* K (<= the weights computed on the source handle) */
  int32_t max_batch;     /* samples per batch (default 4096 when 0) */
  int64_t pool_samples;  /* device staging capacity in sample rows (default 32768 when 0) */
  int32_t fp64_serial;   /* 1: one request per batch, FP64 products (the plain baseline) */
  const double *eigscale;/* [K] multiplies coordinate j (seteigscale); NULL = 1 */
  int32_t pca_workers;   /* full-PCA worker handles (default 1 when 0, at most 8) */
  int64_t pca_budget_bytes; /* device bytes the running PCA jobs may hold (default 64 GiB) */
  int32_t host_loop;     /* 1: the scheduler thread launches each batch's kernels; 0 (default):
                            one device-resident loop (below) forms and runs the batches */
} gp_serve_opts;

int gp_serve_open(gp_ctx *src, const gp_serve_opts *opts, gp_server **out);
/* panel SNP count and bytes per request row */
int gp_serve_layout(const gp_server *srv, int64_t *nsnp, int64_t *row_bytes);
/* [nsnp] genotype SNP record (index into the source handle's loaded SNPs) of each panel SNP */
int gp_serve_panel_snps(const gp_server *srv, int32_t *snp_index);
/* queue a request; *ticket identifies it.  GP_ERR_FULL if it can never fit the pool. */
int gp_serve_submit(gp_server *srv, const uint8_t *codes, int32_t nsamp, double *coords,
                    int32_t *status, int64_t *ticket);
/*
 * Queue a full-PCA job (gp_smartpca_run of gpupca_run.h on panel->records, which must be host
 * records).  Jobs are admitted in FIFO order while the sum of their estimated device
 * footprints (gp_smartpca_footprint) fits pca_budget_bytes (a job is always admitted when no
 * other runs), each on a worker handle with its own stream, so they overlap the projection
 * batches; the worker frees its device memory after each job.  The panel, opts and result
 * arrays must stay valid until the job completes; the ticket works with test/wait.
 */
int gp_serve_submit_pca(gp_server *srv, const gp_panel *panel, const gp_smartpca_opts *opts,
                        gp_run_result *result, int64_t *ticket);
/* device bytes one gp_smartpca_run on nind x nsnp holds at most (an upper estimate) */
int64_t gp_smartpca_footprint(int32_t nind, int64_t nsnp, int32_t precision, int32_t numeigs);
/* PCA jobs completed, the largest number that ran at once, bytes admitted now */
int gp_serve_pca_stats(const gp_server *srv, int64_t *jobs_done, int32_t *peak_running,
                       int64_t *bytes_in_use);
/* the device-resident loop: 1 when it runs (0 with host_loop or fp64_serial), graph launches
 * made (1 per server), batches it ran, polls that ran out with no request published */
int gp_serve_loop_stats(const gp_server *srv, int32_t *device_loop, int64_t *launches,
                        int64_t *batches, int64_t *idle_polls);

/* 1 when the request has completed, 0 while pending, < 0 on error.  A call that reports
 * completion (1 or the request's error) releases the ticket; one waiter per ticket. */
int gp_serve_test(gp_server *srv, int64_t ticket);
/* block until the request completes (GP_OK or its error, releasing the ticket) or timeout_s
 * passes (GP_ERR_TIMEOUT, the ticket stays valid) */
int gp_serve_wait(gp_server *srv, int64_t ticket, double timeout_s);
/* paused = 1: admission and copies go on but no new batch starts (batches in flight
 * finish); it returns once the device-resident loop has stopped.  paused = 0 resumes (and
 * relaunches the loop).  gp_serve_close resumes and drains.  While the loop runs, calls
 * that synchronise the whole device (cudaFree, cudaHostRegister, cudaDeviceSynchronize, by
 * any thread of the process) wait for it: pause the server around them, or open it with
 * host_loop = 1.  Full-PCA jobs of the server stop the loop themselves while they run. */
int gp_serve_pause(gp_server *srv, int32_t paused);
/* counters: batches run, samples projected, requests completed */
int gp_serve_stats(const gp_server *srv, int64_t *batches, int64_t *samples, int64_t *requests);
const char *gp_serve_last_error(const gp_server *srv);
void gp_serve_close(gp_server *srv);

#ifdef __cplusplus
}
#endif
#endif
