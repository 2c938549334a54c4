/*
 * oracle.h -- CPU oracle for the event-reweighting path (TEST INFRASTRUCTURE).
 *
 * This library restates, in plain FP64 C++, GUNDAM's CPU propagation of one
 * likelihood evaluation: the per-event dial product
 * (src/DialDictionary/DialEngine/src/EventDialCache.cpp:156-171), the
 * histogram refill (src/SamplesManager/src/Histogram.cpp:107-135), the
 * per-bin likelihoods (PoissonLogLikelihood.h:19-53,
 * BarlowBeestonBanff2022.h:150-294) and the prior penalty
 * (src/StatisticalInference/Likelihood/src/LikelihoodInterface.cpp:186-215).
 * The per-dial arithmetic follows src/Utils/include/Calculate*.h.
 *
 * It is the checker for the CUDA engine, and its timed runs are the CPU
 * baseline.  Only tests, the smoke check and the benchmark's CPU-baseline leg
 * use it; the engine never calls it.
 */
#ifndef GW_ORACLE_H
#define GW_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_input {
  int32_t n_events, n_params, n_bins, n_samples, n_tables;
  int32_t llh_type;          /* 0 none, 1 Poisson, 2 Barlow-Beeston OA2021 */
  double max_weight;         /* cap on the dial product; <= 0: none */
  const int32_t* event_bin;
  const double* event_w0;
  const int64_t* event_dial_start;
  const uint8_t* dial_type;
  const int32_t* dial_par0;
  const int32_t* dial_par1;
  const int64_t* dial_data_start;
  const double* dial_data;
  const double* mirror_lo;
  const double* mirror_hi;
  const double* clamp_lo;
  const double* clamp_hi;
  const uint8_t* truncate;
  const int32_t* sample_bin_start;
  const double* data;
  const int32_t* table_size;
  const int32_t* table_fn_par;      /* [n_tables*6], -1 = host table */
  const int64_t* table_node_start;
  const double* table_nodes;        /* host tables: values; function tables: energies */
  const double* table_clamp;        /* [n_tables*2] */
  const double* prior_mean;         /* NULL = no penalty */
  const double* prior_icov;
} oracle_input;

typedef struct oracle oracle;

int oracle_create(const oracle_input* in, oracle** out);
int oracle_destroy(oracle* o);

/* K points (row-major K x n_params).  Any output may be NULL.
 *   sums, sums2 [K*n_bins]: sum of w and of w^2 per bin
 *   llh_stat [K], penalty [K]
 *   weights [n_events]: event weights of point 0 */
int oracle_eval(oracle* o, const double* params, int32_t K, int32_t threads, double* sums, double* sums2,
                double* llh_stat, double* penalty, double* weights);

/* One dial response before the response clamp, as the CPU dial class
 * computes it (type = GW_DIAL_*; data in the getDialData() layout).
 * Table dials are not served here. */
double oracle_dial(int32_t type, const double* data, int32_t n_data, double x, double y, int32_t truncate);

/* One bin of the likelihood: type 1 Poisson(data, pred), type 2
 * Barlow-Beeston OA2021(data, pred, sqrt(sum w^2)). */
double oracle_llh_bin(int32_t type, double data, double pred, double sqrt_sum_w2);

#ifdef __cplusplus
}
#endif

#endif
