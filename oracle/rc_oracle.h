/*
 * CPU restatement of RheoCell's time-step hot path -- TEST INFRASTRUCTURE.
 *
 * This library is the checker for the GB300 engine: only tests/, the smoke
 * check and bench.py's CPU-baseline leg load it.  The product never links it.
 * It takes the same inputs as the engine's C ABI (include/rheocell_gb300.h)
 * and restates, serially and in the reference's evaluation order, the
 * functions listed in rc_oracle.c.
 *
 * Parity pin: tests/golden/ holds dumps of the unmodified reference (built by
 * oracle/Makefile, driven by oracle/ref_driver.cpp) that this restatement
 * reproduces; the wet models are pinned against "reference + the project's
 * Eigen-API shim" (oracle/eigen_shim), since Eigen itself is absent.
 */
#ifndef RC_ORACLE_H
#define RC_ORACLE_H

#include "../include/rheocell_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_sim orc_sim;

int orc_create(const rc_params *params, const rc_box *box, int n_cells,
               const rc_cell_host *cells, orc_sim **out);
int orc_step(orc_sim *s, int n_steps, rc_step_stats *stats);
int orc_set_phase(orc_sim *s, int active);
int orc_get_sizes(const orc_sim *s, int *n_cells, int *lsub_x, int *lsub_y);
int orc_download(const orc_sim *s, rc_cell_host *cells, unsigned fields_mask);
long long orc_site_count(const orc_sim *s);
/* drand48 state after the steps run so far (the engine's must match). */
unsigned long long orc_rng_state(const orc_sim *s);
const char *orc_last_error(const orc_sim *s);
void orc_destroy(orc_sim *s);

#ifdef __cplusplus
}
#endif

#endif
