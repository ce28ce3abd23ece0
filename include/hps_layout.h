/*
 * hps_layout.h -- element record layout shared by the C ABI, the Python
 * host layer and the CPU oracle.
 *
 * A beamline element is a type code plus HPS_NPARAM doubles.  The slots
 * follow the setters of the reference's element classes
 * (src/beamline/inc/beamline_element.h:39-263) and, for RF gaps, the field
 * order of RFGapParameter (src/beamline/inc/rfgap_parameter.h:4-32).
 */
#ifndef HPS_LAYOUT_H
#define HPS_LAYOUT_H

#define HPS_NPARAM 32

/* Element type codes.  Names in comments are the reference's type strings
 * (BeamLineElement::GetType). */
enum hps_element_type {
  HPS_ELEM_DRIFT = 1,        /* "Drift"      */
  HPS_ELEM_QUAD = 2,         /* "Quad"       */
  HPS_ELEM_RFGAP_DTL = 3,    /* "RFGap-DTL"  */
  HPS_ELEM_RFGAP_CCL = 4,    /* "RFGap-CCL"  */
  HPS_ELEM_BUNCHER = 5,      /* "Buncher"    */
  HPS_ELEM_STEERER = 6,      /* "Steerer"    */
  HPS_ELEM_APERTURE_C = 7,   /* "ApertureC"  */
  HPS_ELEM_APERTURE_R = 8,   /* "ApertureR"  */
  HPS_ELEM_DIAGNOSTICS = 9,  /* "Diagnostics"*/
  HPS_ELEM_ROTATION = 10,    /* "Rotation"   */
  HPS_ELEM_SPCHCOMP = 11,    /* "SpchComp"   */
  HPS_ELEM_DIPOLE = 12       /* "Dipole"     */
};

/* Slots common to every element. */
#define HPS_P_LENGTH 0   /* [m] */
#define HPS_P_APERTURE 1 /* radius [m], 0 = no aperture */
#define HPS_P_MONITOR 31 /* monitor flag (1 = on) */

/* Quad */
#define HPS_P_GRADIENT 2 /* [T/m] */

/* RF gap (DTL and CCL): slots 2..25 follow RFGapParameter after `length`. */
#define HPS_P_RF_FREQ 2
#define HPS_P_RF_CLBL 3          /* cell_length_over_beta_lambda */
#define HPS_P_RF_AMP 4           /* amplitude [MV/m] */
#define HPS_P_RF_PHASE_REF 5     /* [rad] */
#define HPS_P_RF_PHASE_SHIFT 6   /* [rad] */
#define HPS_P_RF_ENERGY_OUT 7    /* design output energy [MeV] */
#define HPS_P_RF_BETA_CENTER 8
#define HPS_P_RF_DG 9            /* electric-geometric centre shift [m] */
#define HPS_P_RF_T 10
#define HPS_P_RF_TP 11
#define HPS_P_RF_SP 12
#define HPS_P_RF_FIT_BETA_CENTER 13
#define HPS_P_RF_FIT_BETA_MIN 14
#define HPS_P_RF_FIT_T0 15       /* t0..t5 = slots 15..20 */
#define HPS_P_RF_FIT_S1 21       /* s1..s5 = slots 21..25 */

/* Buncher */
#define HPS_P_BUN_ON 2
#define HPS_P_BUN_VOLTAGE 3      /* [MV] */
#define HPS_P_BUN_FREQ 4         /* [MHz] */
#define HPS_P_BUN_PHASE 5        /* [rad] */

/* Steerer */
#define HPS_P_STR_BLH 2          /* integrated field [T m] */
#define HPS_P_STR_BLV 3

/* Apertures */
#define HPS_P_APT_IN 2
#define HPS_P_APT_XL 3
#define HPS_P_APT_XR 4
#define HPS_P_APT_YT 5
#define HPS_P_APT_YB 6

/* Rotation */
#define HPS_P_ROT_ANGLE 2        /* [rad] */

/* Space-charge compensation */
#define HPS_P_SPC_FRACTION 2

/* Dipole (DipoleParameter, src/beamline/inc/dipole_parameter.h) */
#define HPS_P_DIP_RADIUS 2
#define HPS_P_DIP_ANGLE 3
#define HPS_P_DIP_EDGE_IN 4
#define HPS_P_DIP_EDGE_OUT 5
#define HPS_P_DIP_HALF_GAP 6
#define HPS_P_DIP_K1 7
#define HPS_P_DIP_K2 8
#define HPS_P_DIP_FIELD_INDEX 9
#define HPS_P_DIP_KINETIC_ENERGY 10

/* Beam coordinate selectors (order of Beam::{x,xp,y,yp,phi,w,phi_r}). */
#define HPS_COORD_X 0
#define HPS_COORD_XP 1
#define HPS_COORD_Y 2
#define HPS_COORD_YP 3
#define HPS_COORD_PHI 4
#define HPS_COORD_W 5
#define HPS_COORD_PHI_R 6

/* Per-element monitor record (side-effect-free beam statistics written after
 * each simulated element).  Values are what the reference's getters return
 * right after Beam::UpdateLoss (src/pywrapper/src/wrap_beam.cpp:1188-1240). */
#define HPS_MON_NALIVE 0      /* loss == 0 */
#define HPS_MON_NGOOD 1       /* loss == 0 && lloss == 0 */
#define HPS_MON_X_AVG 2
#define HPS_MON_X_SIG 3
#define HPS_MON_XP_AVG 4
#define HPS_MON_XP_SIG 5
#define HPS_MON_X_EMIT 6      /* normalised by beta*gamma of particle 0 */
#define HPS_MON_Y_AVG 7
#define HPS_MON_Y_SIG 8
#define HPS_MON_YP_AVG 9
#define HPS_MON_YP_SIG 10
#define HPS_MON_Y_EMIT 11
#define HPS_MON_PHIR_AVG 12   /* phase relative to particle 0, wrapped */
#define HPS_MON_PHIR_SIG 13
#define HPS_MON_W_AVG 14
#define HPS_MON_W_SIG 15
#define HPS_MON_Z_EMIT 16     /* sqrt(var(phi_r) var(w) - cov^2) [rad MeV] */
#define HPS_MON_W0 17         /* particle 0 kinetic energy */
#define HPS_MON_PHI0 18       /* particle 0 absolute phase */
#define HPS_MON_SC_DR 19      /* SCHEFF mesh dr after the element (0: none) */
#define HPS_MON_SC_DZ 20
#define HPS_MON_SC_REMESH 21  /* number of full SCHEFF solves in the element */
#define HPS_MON_SC_ONMESH 22  /* particles on the mesh at the last solve */
#define HPS_MON_ELEM 23       /* element index */
#define HPS_NMON 24

#endif
