/* Internal entry points used by the reference-signature drop-ins (tm_dropin.c).
 * They act on colony `cid` of a session and keep its Morton order in mind:
 * uploads arrive in caller order and are permuted into slot order, downloads
 * are permuted back. */
#ifndef TM_DROPIN_API_H
#define TM_DROPIN_API_H
#include <stdint.h>
#include "timothy_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* field offsets of the caller's array of structures */
typedef struct {
    int64_t stride;
    int64_t x, y, z, size, young, ctype, phase;   /* -1: absent */
} tmi_aos_layout;

int tmi_set_types(tm_session *s, const tm_celltypes *types);
int tmi_set_dimension(tm_session *s, int dim);
/* caller-order AoS cells (host) -> colony state; n may not exceed the colony's slots */
int tmi_upload_aos(tm_session *s, int cid, const void *cells, int64_t n, const tmi_aos_layout *lay);
/* the same: with the colony's cell count unchanged the cells are taken as
 * the same cells in the same order, keep their slots and (unless one moved
 * too far or changed size or type) the colony's neighbour lists */
int tmi_upload_aos_keep(tm_session *s, int cid, const void *cells, int64_t n, const tmi_aos_layout *lay);
/* largest cell type among the uploaded cells */
int tmi_max_ctype(tm_session *s, int cid, int *maxtype);
/* 0 build (octbuild), 1 pair + octree walk, 2 position update, 3 CIC deposit */
int tmi_phase(tm_session *s, int which);
/* three doubles per cell, caller order, into the host AoS at byte offset `off`:
 * which = 0 -> (v, density, mindist), 1 -> (x, y, z) */
/* pinned: the records are page-locked (the device writes them directly) */
int tmi_download_aos3(tm_session *s, int cid, void *cells, int64_t stride, int64_t off, int which, int pinned);
/* forces as packed (x, y, z) triples in caller order */
int tmi_download_forces(tm_session *s, int cid, double *f3);
int tmi_upload_forces(tm_session *s, int cid, const double *f3);
int tmi_upload_removecell(tm_session *s, int cid, const unsigned char *rem);
int tmi_download_removecell(tm_session *s, int cid, unsigned char *rem, int64_t *newly_marked);
int tmi_set_update(tm_session *s, int cid, int mode, double dt);
/* CIC grid geometry (allocates the colony's grid on first use or change) */
int tmi_set_cic(tm_session *s, int cid, const double lower[3], float res, const int64_t gsize[3]);
/* patch corners of the last deposit and the deposit over [lo, hi] (x-major, z fastest) */
int tmi_patch_box(tm_session *s, int cid, int64_t lo[3], int64_t hi[3]);
int tmi_read_patch(tm_session *s, int cid, const int64_t lo[3], const int64_t hi[3], double *dst);
/* device scratch large enough for n cells of `stride` bytes */
int tmi_reserve_stage(tm_session *s, int64_t bytes);
/* grid -> cell gather from a host patch (fields then gradients) into per-field host arrays */
int tmi_env2cells_patch(tm_session *s, int cid, const double *patch, int nfields, const int64_t box_lo[3],
                        const int64_t box_size[3], const double lower[3], float resolution, const int64_t grid_hi[3],
                        double **cellenv);
/* the random move's rand() values (dim per cell, caller order); NULL clears */
int tmi_set_move_draws(tm_session *s, const int *draws, int64_t count);
/* the same values generated on the device from the C library's generator
 * window w (31 words, oldest first); end receives the window after them */
int tmi_set_move_draws_window(tm_session *s, const uint32_t w[31], int64_t count, uint32_t end[31]);
/* updatecellcycles on host celldata_t records (after tmi_upload_aos of them);
 * counts[0..5]: change of the phase counters, counts[8 + t]: daughters of type t */
int tmi_cycle_aos(tm_session *s, int cid, void *cells, int64_t n, int64_t cap, const tm_cycle_params *p,
                  double *const *cellenv, unsigned char *removecell, int64_t *marked, int64_t *nout,
                  int64_t counts[16]);
/* cellsdeath on host celldata_t records; removed[t * 8 + p]: removed cells of
 * type t in phase p (p = 7 for the necrotic phase) */
int tmi_compact_aos(tm_session *s, void *cells, int64_t n, int64_t oldlnc, const unsigned char *removecell,
                    int64_t *nout, int64_t removed[64]);
/* environment_compute's fields on the device (every field from its mean,
 * the reference's point source); tmi_env_solution reads field f back */
int tmi_env_compute(tm_diffusion *d, int nfields, const double *mean, const double *dc, const double *bc,
                    const double *lambda, float resolution, float secondsperstep, float gfdt, int step,
                    tm_diffusion_stats *stats);
int tmi_env_solution(tm_diffusion *d, int f, double *host);
/* gradient of one field, host arrays */
int tmi_field_gradient_host(tm_session *s, const double *data, const int64_t gsize[3], float resolution,
                            double *gradient);

#ifdef __cplusplus
}
#endif
#endif
