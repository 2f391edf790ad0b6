/*
 * CPU oracle for the pore-throat and shortest-path pipeline of PorousMediaAnalysis.
 *
 * TEST INFRASTRUCTURE ONLY. This library is a sequential CPU restatement of the
 * reference services (the .cpp files of ImageProcessing/Services/Source). It exists to check
 * the CUDA product path; only tests/, __graft_entry__.smoke() and the
 * cpu_baseline leg of bench.py may load it. The product library never links it.
 *
 * Volumes are dense [z][x][y] arrays (y fastest), linear index (z*SX + x)*SY + y,
 * exactly the in-memory order of DataArray (ImageProcessing/Model/Headers/DataArray.h:85-94).
 * Solid voxels are any non-zero byte of the input mask, as in
 * EuclideanDistanceComputer.cpp:167 and ShortestPathComputer.cpp:289.
 */
#ifndef PMA_ORACLE_H
#define PMA_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* One pore row of pores.txt (Serializer.cpp:187-201). */
typedef struct orc_pore {
    uint32_t id;
    int32_t seed_x, seed_y, seed_z;
    uint32_t seed_r2;
    int32_t is_boundary;
    uint64_t volume;
} orc_pore;

/* One shared-pixel-type (throat) row of sharedPixelTypes.txt (Serializer.cpp:203-221).
 * Its pore ids live in the table's pool at [pool_offset, pool_offset + n_pores). */
typedef struct orc_throat {
    uint32_t id;
    uint32_t n_pores;
    uint64_t volume;
    uint64_t pool_offset;
} orc_throat;

/* One line of cavityDescriptions.txt (Serializer.cpp:161-185). */
typedef struct orc_cavity {
    uint32_t id;
    int32_t seed_x, seed_y, seed_z;
    float distance_to_center;
    int32_t reached_walls;
    uint64_t void_count;
    int32_t reaches_all_walls;
    int32_t pad_;
} orc_cavity;

typedef struct orc_table orc_table; /* opaque pores + throats table */

/* a1-a4: squared EDT with the X-only virtual boundary, max EDT^2 and the histogram of
 * non-boundary-crossing balls (EuclideanDistanceComputer.cpp:30-343). hist receives
 * max_edt2+1 counters when hist_cap allows; *hist_len gets max_edt2+1 in any case. */
int orc_edt(const uint8_t* solid, int sx, int sy, int sz, uint32_t* edt2,
            uint32_t* max_edt2, uint64_t* hist, size_t hist_cap, size_t* hist_len);

/* a5-a6: containing-ball radii and coordinates, single-thread semantics
 * (ContainingBallsAssigner.cpp:101-183). */
int orc_containing_balls(const uint32_t* edt2, int sx, int sy, int sz, uint32_t max_edt2,
                         uint32_t* crad2, uint32_t* cx, uint32_t* cy, uint32_t* cz);

/* a7: IsMaximumBall mask (0 solid, 127 inner, 255 outer) and maximum-ball count
 * (ContainingBallsAssigner.cpp:190-250). */
int orc_max_ball_mask(const uint32_t* cx, const uint32_t* cy, const uint32_t* cz,
                      int sx, int sy, int sz, uint8_t* mask, uint64_t* count);

/* a8-a10: sorted maximum balls, pore seeds and the initial DFS propagation
 * (PoreAndThroatComputer.cpp:93-269, BasePoreAndThroatComputer.cpp:37-133).
 * labels must be zeroed by the caller (DataArraysGroup default UNKNOWN_PORE_INDEX). */
orc_table* orc_pores(const uint8_t* mask, const uint32_t* edt2, const uint32_t* crad2,
                     int sx, int sy, int sz, int d3q7, uint32_t* labels);

/* The maximum balls of a8 in std::sort order (linear indices); returns their number. */
size_t orc_sorted_balls(const uint8_t* mask, const uint32_t* edt2, int sx, int sy, int sz,
                        uint32_t* out, size_t cap);

/* a11: empty-pore removal; rewrites the table and remaps labels (EmptyPoresRemover.cpp:31-244). */
int orc_remove_empty_pores(orc_table* t, uint32_t* labels, int sx, int sy, int sz);

/* a12: watershed from the pores of t (WatershedComputer.cpp:80-219). labels_ws zeroed by caller. */
orc_table* orc_watershed(const orc_table* pores_after_removal, const uint32_t* crad2,
                         int sx, int sy, int sz, int d3q7, uint32_t max_edt2, uint32_t* labels_ws);

/* Table accessors. */
size_t orc_table_npores(const orc_table* t);
const orc_pore* orc_table_pores(const orc_table* t);
size_t orc_table_nthroats(const orc_table* t);
const orc_throat* orc_table_throats(const orc_table* t);
size_t orc_table_pool_size(const orc_table* t);
const uint32_t* orc_table_pool(const orc_table* t);
void orc_table_free(orc_table* t);
orc_table* orc_table_from_pores(const orc_pore* pores, size_t n);

/* a13-a15: geodesic distances, cavity ids and cavity descriptions
 * (ShortestPathComputer.cpp:39-511). Returns the number of cavities (the first cav_cap of
 * them are written to cav), or -1 on error. The f64 variant is the FP64 restatement of the same algorithm. */
int orc_geodesic_f32(const uint8_t* solid, int sx, int sy, int sz, int d3q7,
                     float* dist, uint32_t* cavity, orc_cavity* cav, int cav_cap);
int orc_geodesic_f64(const uint8_t* solid, int sx, int sy, int sz, int d3q7,
                     double* dist, uint32_t* cavity, orc_cavity* cav, int cav_cap);

#ifdef __cplusplus
}
#endif
#endif
