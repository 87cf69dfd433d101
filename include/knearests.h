/*
 * knearests.h -- drop-in for the reference's grid kNN API (knearests.h:1-28).
 *
 * Same struct layout for the fields the reference's driver reads
 * (allocated_points, dimx/y/z, d_permutation, d_counters, d_ptrs,
 * d_stored_points, d_knearests; voronoi.cu:1016, 1026, 1061-1062), same
 * ownership (kn_prepare's result is freed by kn_free; kn_get_* return malloc'd
 * host copies the caller frees) and the same failure behaviour (message on
 * stderr, exit(EXIT_FAILURE); knearests.cu:161-164, 205-206, 250-251).
 *
 * Differences, by design:
 *   - the order of points inside a grid cell is by input index, so the
 *     permutation is deterministic (the reference's depends on atomics);
 *   - K is a runtime value (kn_prepare uses 90, the reference's _K_ of
 *     params.h:9; kn_prepare_k takes any 1 <= K <= 128, K < numpoints);
 *   - neighbour lists are ordered by (distance, input index);
 *   - any point count > K works (the reference needs ~12.7k points);
 *   - the cell-offset table is not used: d_cell_offsets, d_cell_offset_dists
 *     and d_cell_max are NULL and num_cell_offsets is 0.
 * The kn_*_ex variants return an error code instead of exiting.
 */
#pragma once

#include <vector_types.h> /* float3 */

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int allocated_points;         /* number of input points                          */
  int dimx, dimy, dimz;         /* grid resolution                                 */
  int num_cell_offsets;         /* 0: no ring-offset table                         */
  int* d_cell_offsets;          /* NULL                                            */
  float* d_cell_offset_dists;   /* NULL                                            */
  float* d_cell_max;            /* NULL                                            */
  unsigned int* d_permutation;  /* sorted position -> input index, numpoints       */
  int* d_counters;              /* points per cell, dimx*dimy*dimz                 */
  int* d_ptrs;                  /* first sorted position of each cell              */
  int* d_globcounter;           /* total number of stored points, 1                */
  float3* d_stored_points;      /* points in grid order, numpoints                 */
  unsigned int* d_knearests;    /* K nearest per point, row-major, sorted space    */
  /* fields below are not in the reference's struct */
  int k;                        /* neighbours per point                            */
  int reserved;
  void* impl;                   /* internal buffers                                */
} kn_problem;

kn_problem* kn_prepare(float3* points, int numpoints);
void kn_solve(kn_problem* kn);
void kn_free(kn_problem** kn);
void kn_print_stats(kn_problem* kn);

float3* kn_get_points(kn_problem* kn);
unsigned int* kn_get_knearests(kn_problem* kn);
unsigned int* kn_get_permutation(kn_problem* kn);

/* Extensions. */
kn_problem* kn_prepare_k(const float3* points, int numpoints, int k);
int kn_prepare_ex(kn_problem** out, const float* points_xyz, int numpoints, int k);
int kn_solve_ex(kn_problem* kn);
int kn_free_ex(kn_problem* kn);

#ifdef __cplusplus
}
#endif
