/*
 * gw_workload.h -- seeded synthetic event/dial workloads (libgw_workload.so).
 *
 * GUNDAM builds its event/dial cache from ROOT trees and a YAML/JSON
 * configuration (DataDispenser.cpp:733, DialCollection.cpp).  No such inputs
 * exist here, so this generator draws events, dials, binning, a data
 * histogram and a prior with the shapes of the five benchmark
 * configurations, in the neutral event-major form an EventDialCache holds:
 * every event owns a list of dials, each dial carries the data vector its
 * DialBase::getDialData() would return (formats as in gw.h).
 *
 * Generation is deterministic for a given (config, seed, n_events): each
 * event draws from its own counter-seeded stream, so the result does not
 * depend on the number of threads.
 */
#ifndef GW_WORKLOAD_H
#define GW_WORKLOAD_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Benchmark configurations. */
enum {
  GWW_C1 = 1, /* 100k events, 3 monotonic + 2 norm dials, 20x20 bins, Poisson   */
  GWW_C2 = 2, /* 5M events, Poisson(8) mixed dials, 8 samples / 3000 bins, BB    */
  GWW_C5 = 5, /* 40M events, Poisson(10) spline/graph dials + 1 kriged, 10k bins */
  GWW_MIXED_SMALL = 9 /* every dial type incl. compact/bicubic/tabulated, mirrors,
                         truncation, cap: a small case for parity edge tests */
};

typedef struct gww_workload {
  int32_t config;
  int32_t n_events;
  int32_t n_params;
  int32_t n_bins;
  int32_t n_samples;
  int32_t n_tables;
  int64_t n_dials;
  int64_t n_data;
  double max_weight;          /* event-weight cap on the dial product, <= 0: none */

  /* events */
  int32_t* event_bin;         /* [n_events] global bin */
  double* event_w0;           /* [n_events] base weight */
  int64_t* event_dial_start;  /* [n_events + 1] */
  /* dials, event-major */
  uint8_t* dial_type;         /* [n_dials] GW_DIAL_* */
  int32_t* dial_par0;         /* [n_dials] (-1 for table dials) */
  int32_t* dial_par1;         /* [n_dials] (-1 unless surface) */
  int64_t* dial_data_start;   /* [n_dials + 1] */
  double* dial_data;          /* [n_data] */
  /* parameters */
  double* mirror_lo;          /* [n_params] -DBL_MAX when unused */
  double* mirror_hi;          /* [n_params] +DBL_MAX when unused */
  double* clamp_lo;           /* [n_params] response clamp of the parameter's dials */
  double* clamp_hi;           /* [n_params] */
  uint8_t* truncate;          /* [n_params] 1 = allowDialExtrapolation false */
  double* prior_mean;         /* [n_params] */
  double* prior_cov;          /* [n_params * n_params] */
  /* histogram */
  int32_t* sample_bin_start;  /* [n_samples + 1] */
  double* data;               /* [n_bins] observed counts */
  /* tables */
  int32_t* table_size;        /* [n_tables] */
  int32_t* table_fn_par;      /* [n_tables * 6] parameters of the oscillation function, -1 = host table */
  int64_t* table_node_start;  /* [n_tables + 1] */
  double* table_nodes;        /* node energies (function tables) or values (host tables) */
  double* table_clamp;        /* [n_tables * 2] */
} gww_workload;

/* n_events <= 0 keeps the configuration's own event count. threads <= 0 uses
 * all host cores. */
int gww_create(int32_t config, int64_t n_events, uint64_t seed, int32_t threads, gww_workload** out);
int gww_destroy(gww_workload* w);
const char* gww_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* GW_WORKLOAD_H */
