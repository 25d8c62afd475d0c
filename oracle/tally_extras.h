/* Per-ray statistics derived from one ray record (test infrastructure only).
 *
 * Restates the reference host's per-chunk numpy reductions of simulate()
 * (CLARITAS/CLARITAS.py:8483-8508 failure subcodes, :8665-8735 entered-ray
 * sums, predicate counts and the interaction-count histogram) for one ray, so
 * the CPU oracles and the reference drivers fill the same clr_tallies fields
 * the library's kernel fills.
 */
#ifndef CLARITAS_TALLY_EXTRAS_H
#define CLARITAS_TALLY_EXTRAS_H

#include <math.h>
#include "claritas_gb.h"

static inline void clr_tally_add_ray_stats(clr_tallies* T, const clr_ray_record* r) {
    if (r->failure_code != 0) T->failure_subcode_counts[CLR_SUBCODE_INDEX(r->failure_subcode)]++;
    const int st = r->status;
    if (st != 3) {
        T->ray_flags[CLR_RF_SOURCE_ACCEPTED]++;
        if (r->source_bore_reflections == 0) T->ray_flags[CLR_RF_SOURCE_DIRECT]++;
        else T->ray_flags[CLR_RF_SOURCE_REFLECTED]++;
    }
    if (st == 1 && isfinite(r->air_x) && isfinite(r->air_vx)) T->ray_flags[CLR_RF_VALID_AIR]++;
    if (st == 8) T->ray_flags[CLR_RF_TRAPPED]++;
    if (r->entered_water > 0) {
        T->ray_flags[CLR_RF_ENTERED]++;
        if (r->interaction_count == 0) T->ray_flags[CLR_RF_BALLISTIC]++;
        if (r->entry_reflections > 0) T->ray_flags[CLR_RF_ENTRY_REFLECTED]++;
        if (r->internal_reflections > 0) T->ray_flags[CLR_RF_INTERNAL_REFLECTED]++;
        if (r->absorptions > 0) T->ray_flags[CLR_RF_ABSORBED]++;
        if (r->cell_tir > 0) T->ray_flags[CLR_RF_CELL_TIR]++;
        if (r->top_tir > 0) T->ray_flags[CLR_RF_TOP_TIR]++;
        if (r->bottom_tir > 0) T->ray_flags[CLR_RF_BOTTOM_TIR]++;
        const int32_t v[16] = {r->interaction_count, r->geometric, r->wave, r->coherent, r->morphology,
                               r->particle_reflections, r->cell_inner_reflections, r->cell_outer_reflections,
                               r->top_reflections, r->bottom_inner_reflections, r->bottom_outer_reflections,
                               r->cell_tir, r->top_tir, r->bottom_tir, r->entry_reflections, r->internal_reflections};
        for (int k = 0; k < 16; ++k) T->entered_sums[k] += v[k];
        int ic = r->interaction_count;
        if (ic < 0) ic = 0;
        if (ic > CLR_IC_HIST - 1) ic = CLR_IC_HIST - 1;
        T->ic_hist[ic]++;
    }
}

static inline void clr_tally_merge_extras(clr_tallies* dst, const clr_tallies* src) {
    for (int k = 0; k < 16; ++k) { dst->entered_sums[k] += src->entered_sums[k]; dst->ray_flags[k] += src->ray_flags[k]; }
    for (int k = 0; k < CLR_N_SUBCODES; ++k) dst->failure_subcode_counts[k] += src->failure_subcode_counts[k];
    for (int k = 0; k < CLR_IC_HIST; ++k) dst->ic_hist[k] += src->ic_hist[k];
}

#endif
