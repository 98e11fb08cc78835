/* btegpu_debug.h - host-only views of the engine's tables, exported for the
 * CPU test suite (no GPU needed).  Not part of the public ABI. */
#ifndef BTEGPU_DEBUG_H
#define BTEGPU_DEBUG_H

#include "../../include/btegpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Per box: nborders, (p1x p1y p2x p2y npx npy) per border, ncontacts,
 * (id npx npy) per contact, centre x, y, area.  Returns the count written
 * (or needed when above cap), -1 on error. */
long long btegpu_debug_geometry(const bte_geometry* g, double* out, long long cap);

/* 1 when the boxes tile an axis-aligned grid (fast path), 0 if not. */
int btegpu_debug_grid(const bte_geometry* g, int* nx, int* ny);

/* Lambert-table entries per wall-normal class; returns the total. */
long long btegpu_debug_lambert(const bte_mode_table* m, const bte_geometry* g,
                               long long* nnz_per_class, int maxclass);

/* One properties.msgpack.bin frame; returns its byte count. */
long long btegpu_debug_frame(double time, double Eeff, const double* temps, const int* H, int nboxes,
                             int nmodes, char* out, long long cap);

/* The host build of bte_log. */
int btegpu_debug_log(const double* x, double* y, long long n);

#ifdef __cplusplus
}
#endif

#endif
