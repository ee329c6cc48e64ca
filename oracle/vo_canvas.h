/*
 * vo_canvas — CPU restatement of the reference's Canvas
 * (src/voromesh/canvas.cpp, include/voromesh/canvas.h).
 *
 * TEST INFRASTRUCTURE ONLY: loaded by the tests and by bench.py's CPU leg as
 * the checker, never by the product library.
 *
 * Same voxel/tile layout, float arithmetic in the reference's order and
 * double per-voxel sums in sample order. One deliberate difference: the
 * reference visits a stamp's rim voxels in std::unordered_map order
 * (canvas.cpp:200), which only decides which of the slots popped from the
 * free list goes to which rim voxel. Here rim voxels are visited in tile-major
 * order (tile row, tile column, bit), the order RasterizeShape uses
 * (canvas.cpp:102-106). States therefore agree with the reference's up to a
 * relabelling of slot indices; everything else (occupancy, surface masks and
 * points, slot values, free-list length, edit counts) is identical.
 */
#ifndef VO_CANVAS_H
#define VO_CANVAS_H

#include <stdint.h>

#include "vm_oracle.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct vo_canvas vo_canvas;

typedef struct {
    int tx0, ty0, tx1, ty1; /* occupancy tiles [tx0,tx1) x [ty0,ty1) rewritten */
    int removed, added, flipped;
    int ndirty;
} vo_canvas_edit;

vo_canvas *vo_canvas_create(float width, float height, float voxelSize);
void vo_canvas_destroy(vo_canvas *c);
/* Canvas::RasterizeShape (canvas.cpp:71-134); 0 on success */
int vo_canvas_rasterize(vo_canvas *c, const vo_f2 *poly, int n);
/* Canvas::StampDisc (canvas.cpp:136-221) */
int vo_canvas_stamp(vo_canvas *c, float cx, float cy, float radius, int inside, vo_canvas_edit *e);
/* dims: voxelsX, voxelsY, tilesX, tilesY */
void vo_canvas_dims(const vo_canvas *c, int *dims);
/* counts: slots, free slots, surface voxels, surface tiles */
void vo_canvas_counts(const vo_canvas *c, long long *counts);
/* Any pointer may be NULL. spt/sslot are dense (tiles x 64, tile-major);
 * voxels off the surface read (-1,-1) / -1. dirty = the last edit's list. */
void vo_canvas_get(const vo_canvas *c, vo_f2 *slots, int *freeList, uint64_t *inside, uint64_t *smask, vo_f2 *spt,
                   int *sslot, int *dirty);

#ifdef __cplusplus
}
#endif

#endif
