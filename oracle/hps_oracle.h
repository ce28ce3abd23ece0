/*
 * hps_oracle.h -- FP64 CPU restatement of HPSim's per-element tracking path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the oracle the CUDA
 * implementation in hpsim_gb300/ is tested against: it is loaded by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg, never by the
 * product.  Every routine cites the reference file:line it restates.
 *
 * Parity pin: the restatement is compared against the reference's own kernel
 * sources compiled for the host (oracle/ref_harness.cpp, built into
 * oracle/_ref/ when the reference tree is present) and against the golden
 * fixtures generated from that build (tests/golden/).
 */
#ifndef HPS_ORACLE_H
#define HPS_ORACLE_H

#include <stdint.h>
#include "../include/hps_layout.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Indices into orc_beam.st (the reference's per-beam device scalars,
 * src/beam/inc/beam.h:175-256). */
enum {
  ORC_X_AVG, ORC_X_AVG_GOOD, ORC_XP_AVG, ORC_Y_AVG, ORC_Y_AVG_GOOD, ORC_YP_AVG,
  ORC_PHI_AVG, ORC_PHI_AVG_R, ORC_PHI_AVG_GOOD, ORC_W_AVG, ORC_W_AVG_GOOD,
  ORC_X_SIG, ORC_X_SIG_GOOD, ORC_XP_SIG, ORC_Y_SIG, ORC_Y_SIG_GOOD, ORC_YP_SIG,
  ORC_PHI_SIG, ORC_PHI_SIG_R, ORC_PHI_SIG_GOOD, ORC_W_SIG, ORC_W_SIG_GOOD,
  ORC_X_EMIT, ORC_Y_EMIT, ORC_Z_EMIT, ORC_R_MAX, ORC_ABS_PHI_MAX,
  ORC_NSTAT
};

typedef struct orc_beam {
  uint32_t n;
  double mass, charge, current, freq, design_w;
  uint32_t grid_size, blck_size;
  double *x, *xp, *y, *yp, *phi, *phi_r, *w;
  uint32_t *loss, *lloss;
  double st[ORC_NSTAT];
  uint32_t num_loss, num_lloss, num_good;
  /* saved copies: [0] initial, [1] intermediate (beam.cpp:547-647) */
  double *save[2][6];
  uint32_t *save_loss[2], *save_lloss[2];
  double save_design_w[2], save_freq[2], save_current[2];
} orc_beam;

typedef struct orc_scheff {
  uint32_t nx, nz, nx_init, nz_init, adj_bunch;
  double fraction, interval, interval_init, adj_bunch_w, mesh_w;
  double sigr_old, sigz_old, gm_old;
  uint32_t good_cnt_old;
  double remesh_val;
  /* device globals of space_charge_kernel.cu:12-15 */
  double dr, dz;
  uint32_t num_on_mesh;
  double *bin;   /* nz*nx */
  double *fld1;  /* (nx+1)*nx*nz*2 (x,y interleaved) */
  double *fld2;  /* (nz+1)*(nx+1)*2 */
  /* launcher globals of space_charge.cu:16-25 */
  double beta, sc_freq, frac;
  uint32_t adj_cur;
  /* counters for the monitor record */
  uint32_t n_solves;
} orc_scheff;

typedef struct orc_sim {
  orc_beam *beam;
  orc_scheff *spch;            /* may be NULL */
  uint32_t nelem;
  const int *types;            /* nelem */
  const double *params;        /* nelem * HPS_NPARAM */
  int sc_on;
  /* engine globals of simulation_engine.cu:19-33 */
  uint32_t cur_id, ccl_cell_num;
  double design_w, wavelen;
  int prev_end;
  /* optional monitor output: nelem * HPS_NMON doubles */
  double *mon;
  int error;                   /* nonzero after a malformed lattice */
} orc_sim;

/* beam */
orc_beam *orc_beam_create(uint32_t n, double mass, double charge, double current);
void orc_beam_free(orc_beam *b);
void orc_beam_set_distribution(orc_beam *b, const double *x, const double *xp,
    const double *y, const double *yp, const double *phi, const double *w,
    const uint32_t *loss, const uint32_t *lloss);
void orc_beam_set_waterbag(orc_beam *b, double ax, double bx, double ex,
    double ay, double by, double ey, double az, double bz, double ez,
    double sync_phi, double sync_w, double freq, uint32_t seed);
void orc_beam_set_dc(orc_beam *b, double ax, double bx, double ex, double ay,
    double by, double ey, double dphi, double sync_phi, double sync_w,
    uint32_t seed);
void orc_beam_set_ref_w(orc_beam *b, double w);
void orc_beam_set_ref_phi(orc_beam *b, double phi);
void orc_beam_save(orc_beam *b, int slot);
int orc_beam_restore(orc_beam *b, int slot);
void orc_beam_update_loss(orc_beam *b);
void orc_beam_update_longitudinal_loss(orc_beam *b);
void orc_beam_update_good_count(orc_beam *b);
void orc_beam_update_avg(orc_beam *b, int coord, int good_only);
void orc_beam_update_sig(orc_beam *b, int coord, int good_only);
void orc_beam_update_emittance(orc_beam *b);
void orc_beam_update_relative_phi(orc_beam *b, int use_good);
void orc_beam_update_stat_for_sc(orc_beam *b);
void orc_beam_update_avg_xy(orc_beam *b);
void orc_beam_update_max_r_phi(orc_beam *b);
void orc_beam_change_frequency(orc_beam *b, double freq);
void orc_beam_apply_cut(orc_beam *b, char coord, double lo, double hi);
void orc_beam_shift(orc_beam *b, int coord, double val);
void orc_beam_monitor(const orc_beam *b, double *out /* HPS_NMON */);

/* SCHEFF */
orc_scheff *orc_scheff_create(uint32_t nr, uint32_t nz, uint32_t adj_bunch);
void orc_scheff_free(orc_scheff *s);
void orc_scheff_set_interval(orc_scheff *s, double v);
void orc_scheff_set_mesh_size(orc_scheff *s, uint32_t nr, uint32_t nz);
void orc_scheff_start(orc_scheff *s, orc_beam *b, double length);
/* the three mesh stages on their own, for table-level known-answer tests */
void orc_scheff_green_table(orc_scheff *s, double beta, double freq,
    uint32_t num_part, double current_ov_mc2, uint32_t adj_bunch);
void orc_scheff_deposit(orc_scheff *s, const orc_beam *b, double beta, double freq);
void orc_scheff_contract(orc_scheff *s);

/* engine */
orc_sim *orc_sim_create(orc_beam *b, uint32_t nelem, const int *types,
    const double *params, orc_scheff *spch);
void orc_sim_free(orc_sim *s);
void orc_sim_reset(orc_sim *s);
int orc_sim_simulate(orc_sim *s, int start, int end);
void orc_sim_set_monitor(orc_sim *s, double *mon);

int orc_num_threads(void);
void orc_set_threads(int n);

#ifdef __cplusplus
}
#endif
#endif
