"""Element records and the synthetic lattices/beams used for benchmarking.

An element is ``(type, name, params)`` where ``params`` is a float64 array of
``HPS_NPARAM`` slots laid out as in ``include/hps_layout.h``.  The builders
below create the reference's element kinds (src/beamline/inc/beamline_element.h)
without a lattice database, plus three synthetic lattices of the shapes the
benchmarks are quoted on:

* ``small_fodo``: buncher + 40 alternating 0.10 m drifts / 0.05 m quads
  (+-18 T/m), 65,536 particles, SCHEFF 32x128 after every element, FP64.
* ``dtl_like``: 165 DTL RF gaps (E0 = 2.5 MV/m, phi_s = -26 deg) between 0.04 m
  quads (+-80 T/m: at +-45 T/m the zero-current phase advance at 0.75 MeV is
  ~10 deg per period and the 15 mA beam is lost; +-80 T/m gives 60-80 deg and
  a stable beam through all 331 elements); the cell lengths and RF phase
  offsets come from tracking
  the synchronous particle through the gap formulas of
  src/simulation/inc/simulation_kernel.cu:226-497 (on axis, FP64).
* ``ccl_like``: 805 MHz coupled-cavity gaps from 100 MeV with doublets.

The synchronous-particle design here is lattice *design*, not the tracking
path: it fixes the set points (energy_out, phase_shift, cell length) a real
lattice database would hold.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

CLIGHT = 299.792458
NPARAM = 32

DRIFT, QUAD, RFGAP_DTL, RFGAP_CCL, BUNCHER, STEERER = 1, 2, 3, 4, 5, 6
APERTURE_C, APERTURE_R, DIAGNOSTICS, ROTATION, SPCHCOMP, DIPOLE = 7, 8, 9, 10, 11, 12

TYPE_NAMES = {
    DRIFT: "Drift", QUAD: "Quad", RFGAP_DTL: "RFGap-DTL", RFGAP_CCL: "RFGap-CCL",
    BUNCHER: "Buncher", STEERER: "Steerer", APERTURE_C: "ApertureC",
    APERTURE_R: "ApertureR", DIAGNOSTICS: "Diagnostics", ROTATION: "Rotation",
    SPCHCOMP: "SpchComp", DIPOLE: "Dipole",
}
TYPE_CODES = {v.lower(): k for k, v in TYPE_NAMES.items()}

# slot numbers (include/hps_layout.h)
P_LENGTH, P_APERTURE, P_MONITOR = 0, 1, 31
P_GRADIENT = 2
RF_SLOTS = ["frequency", "cell_length_over_beta_lambda", "amplitude", "phase_ref",
            "phase_shift", "energy_out", "beta_center", "dg", "t", "tp", "sp",
            "fit_beta_center", "fit_beta_min", "fit_t0", "fit_t1", "fit_t2", "fit_t3",
            "fit_t4", "fit_t5", "fit_s1", "fit_s2", "fit_s3", "fit_s4", "fit_s5"]
SLOTS = {
    DRIFT: {},
    QUAD: {"gradient": 2},
    RFGAP_DTL: {k: 2 + i for i, k in enumerate(RF_SLOTS)},
    RFGAP_CCL: {k: 2 + i for i, k in enumerate(RF_SLOTS)},
    BUNCHER: {"on": 2, "voltage": 3, "frequency": 4, "phase": 5},
    STEERER: {"blh": 2, "blv": 3},
    APERTURE_C: {"in": 2},
    APERTURE_R: {"in": 2, "xl": 3, "xr": 4, "yt": 5, "yb": 6},
    DIAGNOSTICS: {},
    ROTATION: {"angle": 2},
    SPCHCOMP: {"fraction": 2},
    DIPOLE: {"radius": 2, "angle": 3, "edge_in": 4, "edge_out": 5, "half_gap": 6,
             "k1": 7, "k2": 8, "field_index": 9, "kinetic_energy": 10},
}
COMMON = {"length": P_LENGTH, "aperture": P_APERTURE, "monitor": P_MONITOR}


def element(etype, name: str, **kw):
    """Return ``(type_code, name, params)`` for one beamline element.

    ``etype`` is a type code or the reference's type string ("Quad", ...).
    Keyword names are the reference's setter names in snake case.  Apertures
    and bunchers default to in/on, unlike the reference's constructors, since
    an element added here is meant to act.
    """
    code = TYPE_CODES[etype.lower()] if isinstance(etype, str) else int(etype)
    p = np.zeros(NPARAM, dtype=np.float64)
    slots = dict(COMMON)
    slots.update(SLOTS[code])
    if code in (APERTURE_C, APERTURE_R):
        p[2] = 1.0
    if code == BUNCHER:
        p[2] = 1.0
    if code in (RFGAP_DTL, RFGAP_CCL):
        p[slots["cell_length_over_beta_lambda"]] = 1.0
    for k, v in kw.items():
        if k not in slots:
            raise ValueError(f"{TYPE_NAMES[code]} has no parameter '{k}'")
        p[slots[k]] = float(v)
    return code, name, p


def param_index(etype: int, key: str) -> int:
    slots = dict(COMMON)
    slots.update(SLOTS[etype])
    return slots[key]


# ---------------------------------------------------------------- kinematics
def gamma_of(w, mass):
    return w / mass + 1.0


def beta_of(w, mass):
    g = w / mass
    return math.sqrt(g * (g + 2.0)) / (g + 1.0)


def betagamma_of(w, mass):
    g = w / mass
    return math.sqrt(g * (g + 2.0))


def wrap_pi(a):
    return (a + math.pi) % (2.0 * math.pi) - math.pi


# ------------------------------------------------------------------ beams
@dataclass
class BeamSpec:
    num: int
    mass: float = 939.294
    charge: float = -1.0
    current: float = 0.015
    freq: float = 201.25
    w0: float = 0.750
    phi0: float = 0.0
    seed: int = 12345
    # waterbag arguments of Beam::InitWaterbagBeam (cm/rad, cm*rad total)
    twiss: tuple = field(default_factory=tuple)


def waterbag_twiss(mass=939.294, w0=0.750, freq=201.25, eps_n_rms_cm_mrad=0.02,
                   beta_xy_cm=20.0, eps_z_rms_deg_mev=0.1, beta_z_cm=25.0):
    """Waterbag arguments (ax, bx, ex, ay, by, ey, az, bz, ez) from rms values.

    Transverse: normalised rms emittance [cm mrad] -> unnormalised total
    emittance [cm rad] (divide by beta*gamma and 1000, times 8: for a uniform
    6-ball each coordinate has <r_i^2> = 1/8).  Longitudinal: rms emittance in
    deg MeV converted to the z-z' plane of the waterbag generator
    (z [cm] = phi [deg] * beta*lambda[cm] / 360, z' = dW / (2 W)).
    """
    bg = betagamma_of(w0, mass)
    ex = eps_n_rms_cm_mrad / bg / 1000.0 * 8.0
    bl_cm = beta_of(w0, mass) * CLIGHT / freq * 100.0
    ez = eps_z_rms_deg_mev * (bl_cm / 360.0) / (2.0 * w0) * 8.0
    return (0.0, beta_xy_cm, ex, 0.0, beta_xy_cm, ex, 0.0, beta_z_cm, ez)


def beam_spec(num, seed=12345):
    return BeamSpec(num=num, seed=seed, twiss=waterbag_twiss())


# --------------------------------------------------------------- lattices
def small_fodo(aperture=0.0):
    """Buncher + 40 elements of alternating 0.10 m drifts and 0.05 m quads.

    The buncher has E0T*L = 0.15 MV at phi_s = -90 deg and 201.25 MHz (its
    T(beta) = 1 - 0.4 (beta - 0.04)/0.04 is ~1 at beta ~ 0.04, and the
    reference's buncher has no transit-time factor, so the voltage carries
    E0T*L)."""
    elems = [element(BUNCHER, "BUNCHER01", voltage=0.15, frequency=201.25,
                     phase=math.radians(-90.0), aperture=aperture)]
    for k in range(20):
        elems.append(element(DRIFT, f"DR{k:02d}", length=0.10, aperture=aperture))
        g = 18.0 if k % 2 == 0 else -18.0
        elems.append(element(QUAD, f"QM{k:02d}", length=0.05, gradient=g, aperture=aperture))
    return elems


@dataclass
class ScanBeam:
    """One beam of a batched scan: its particle count, seed and set-point
    perturbations of the small-FODO lattice."""
    num: int
    seed: int
    rf_scale: float      # buncher voltage scale
    phase_offset: float  # buncher phase offset, rad
    quad_scale: float    # scale of every quad gradient


def batched_scan(n_beams=256, seed=2024, n_min=16384, n_max=524288):
    """Independent beams on the small-FODO topology: particle counts
    log-uniform in [n_min, n_max], RF amplitude scale U(0.95, 1.05), phase
    offset U(-3, +3) deg and quad-gradient scale U(0.97, 1.03), from a seed."""
    rng = np.random.default_rng(seed)
    nums = np.exp(rng.uniform(math.log(n_min), math.log(n_max), n_beams)).astype(np.int64)
    out = []
    for k in range(n_beams):
        out.append(ScanBeam(int(nums[k]), int(seed * 1000 + k), float(rng.uniform(0.95, 1.05)),
                            float(math.radians(rng.uniform(-3.0, 3.0))), float(rng.uniform(0.97, 1.03))))
    return out


def scan_lattice(sb: ScanBeam, aperture=0.0):
    """small_fodo with one scan beam's set points."""
    elems = small_fodo(aperture)
    out = []
    for code, name, p in elems:
        p = p.copy()
        if code == BUNCHER:
            p[param_index(BUNCHER, "voltage")] *= sb.rf_scale
            p[param_index(BUNCHER, "phase")] += sb.phase_offset
        elif code == QUAD:
            p[param_index(QUAD, "gradient")] *= sb.quad_scale
        out.append((code, name, p))
    return out


def partition_beams(nums, ranks):
    """Beam indices per rank, balanced by particle count: the largest beams
    first, each to the rank with the fewest particles so far (ties to the
    lower rank); every beam goes to exactly one rank."""
    load = [0] * ranks
    out = [[] for _ in range(ranks)]
    for i in sorted(range(len(nums)), key=lambda k: (-nums[k], k)):
        r = min(range(ranks), key=lambda q: (load[q], q))
        out[r].append(i)
        load[r] += nums[i]
    return [sorted(o) for o in out]


def perturbed_beams(n_beams, num, seed):
    """Equal beams with perturbed set points: RF amplitude scale U(0.99,
    1.01), RF phase offset U(-1, +1) deg and quad-gradient scale U(0.97,
    1.03) per beam."""
    rng = np.random.default_rng(seed)
    return [ScanBeam(num=num, seed=int(rng.integers(1, 2 ** 31)), rf_scale=float(rng.uniform(0.99, 1.01)),
                     phase_offset=math.radians(float(rng.uniform(-1.0, 1.0))),
                     quad_scale=float(rng.uniform(0.97, 1.03))) for _ in range(n_beams)]


def ccl_batch(n_beams=16, num=1 << 20, seed=805):
    """Beams of the CCL-like lattice with perturbed set points (perturbed_beams)."""
    return perturbed_beams(n_beams, num, seed)


def dtl_batch(n_beams=8, num=1 << 20, seed=2025):
    """Beams of the DTL-like lattice with perturbed set points (perturbed_beams)."""
    return perturbed_beams(n_beams, num, seed)


def perturbed(elems, sb: ScanBeam):
    """A lattice with one batch beam's set points: every RF gap's amplitude
    scaled and phase shifted, the buncher's voltage and phase likewise, every
    quad gradient scaled."""
    out = []
    for code, name, p in elems:
        p = p.copy()
        if code in (RFGAP_DTL, RFGAP_CCL):
            p[param_index(code, "amplitude")] *= sb.rf_scale
            p[param_index(code, "phase_shift")] += sb.phase_offset
        elif code == BUNCHER:
            p[param_index(BUNCHER, "voltage")] *= sb.rf_scale
            p[param_index(BUNCHER, "phase")] += sb.phase_offset
        elif code == QUAD:
            p[param_index(QUAD, "gradient")] *= sb.quad_scale
        out.append((code, name, p))
    return out


def _ttf_fit(rng, beta_g, t_nom=0.85, s_nom=0.10, spread=0.05):
    """Cubic T(beta), S(beta) in powers of beta.

    Written in u = (beta - beta_g)/beta_g with nominal coefficients
    T: (0.85, 0.40, -1.2, 0.5), S: (0.10, -0.10, 0.3, -0.1), each drawn
    uniformly within +-5 %, then expanded into powers of beta."""
    tn = np.array([t_nom, 0.40, -1.2, 0.5]) * rng.uniform(1 - spread, 1 + spread, 4)
    sn = np.array([s_nom, -0.10, 0.3, -0.1]) * rng.uniform(1 - spread, 1 + spread, 4)

    def expand(c):
        # sum_k c_k ((beta - bg)/bg)^k  ->  power basis in beta
        out = np.zeros(6)
        for k, ck in enumerate(c):
            poly = np.poly1d([1.0 / beta_g, -1.0]) ** k
            coeffs = poly.coeffs[::-1]
            out[:len(coeffs)] += ck * coeffs
        return out

    return expand(tn), expand(sn)


def _ttf_eval(ta, sa, beta, beta_g, beta_min):
    b = beta
    if beta > 1.1 * beta_g:
        b = beta_g
    elif beta < beta_min:
        b = beta_min
    t = ta[0] + b * (ta[1] + b * (ta[2] + b * (ta[3] + b * (ta[4] + b * ta[5]))))
    coef = b * b / (2.0 * math.pi * beta_g)
    tp = coef * (ta[1] + b * (2 * ta[2] + b * (3 * ta[3] + b * (4 * ta[4] + 5 * b * ta[5]))))
    sp = -coef * (sa[1] + b * (2 * sa[2] + b * (3 * sa[3] + b * (4 * sa[4] + 5 * b * sa[5]))))
    return t, tp, sp


def dtl_like(n_gaps=165, e0=2.5, phi_s_deg=-26.0, quad_len=0.04, grad=80.0,
             w0=0.750, phi0=0.0, freq=201.25, mass=939.294, charge=-1.0, seed=2024,
             aperture=0.0):
    """Quad, gap, quad, gap, ..., quad: ``n_gaps`` DTL gaps, ``n_gaps + 1``
    quads.  Returns the element list; cell lengths grow with the synchronous
    energy."""
    rng = np.random.default_rng(seed)
    lam = CLIGHT / freq
    phi_s = math.radians(phi_s_deg)
    q = abs(charge)
    elems = []
    w, phi = w0, phi0
    for k in range(n_gaps + 1):
        g = grad if k % 2 == 0 else -grad
        elems.append(element(QUAD, f"Q{k:03d}", length=quad_len, gradient=g, aperture=aperture))
        # both quad halves advance the synchronous phase (on axis)
        phi += 2.0 * math.pi * quad_len / (lam * beta_of(w, mass))
        if k == n_gaps:
            break
        beta_in = beta_of(w, mass)
        cell = beta_in * lam
        for _ in range(4):
            bg_ = cell / lam
            ta, sa = _ttf_fit(np.random.default_rng(seed * 1000 + k), bg_)
            t, _, _ = _ttf_eval(ta, sa, beta_in, bg_, 0.5 * bg_)
            dw = q * e0 * cell * t * math.cos(phi_s)
            cell = beta_of(w + 0.5 * dw, mass) * lam
        beta_g = cell / lam
        ta, sa = _ttf_fit(np.random.default_rng(seed * 1000 + k), beta_g)
        t, tp, sp = _ttf_eval(ta, sa, beta_in, beta_g, 0.5 * beta_g)
        # first half: pi*clbl, minus the half quad the previous quad already added
        phi += math.pi - math.pi * quad_len / (beta_in * lam)
        phase_shift = wrap_pi(phi_s - phi)
        dw = q * e0 * cell * t * math.cos(phi_s)
        w_out = w + dw
        beta_out = beta_of(w_out, mass)
        # second half: pi*clbl, minus the following quad's first half
        phi += math.pi - math.pi * quad_len / (beta_out * lam)
        gap_len = cell - quad_len
        kw = dict(length=gap_len, frequency=freq, cell_length_over_beta_lambda=1.0,
                  amplitude=e0, phase_ref=phi_s, phase_shift=phase_shift,
                  energy_out=w_out, beta_center=beta_g, dg=0.0, t=t, tp=tp, sp=sp,
                  fit_beta_center=beta_g, fit_beta_min=0.5 * beta_g, aperture=aperture)
        for j in range(6):
            kw[f"fit_t{j}"] = ta[j]
        for j in range(1, 6):
            kw[f"fit_s{j}"] = sa[j]
        elems.append(element(RFGAP_DTL, f"G{k:03d}", **kw))
        w = w_out
    _ = rng
    return elems


def ccl_like(modules=4, tanks=32, cells=8, e0=1.2, phi_s_deg=-30.0, w0=100.0,
             phi0=0.0, freq=805.0, mass=939.294, charge=-1.0, quad_len=0.08, grad=20.0,
             seed=805):
    """Coupled-cavity gaps: modules x tanks x cells RFGap-CCL elements, a
    doublet of quads (+grad, -grad) and a short drift between tanks."""
    lam = CLIGHT / freq
    phi_s = math.radians(phi_s_deg)
    q = abs(charge)
    elems = []
    w, phi = w0, phi0
    n = 0
    for mod in range(modules):
        for tk in range(tanks):
            for c in range(cells):
                beta_in = beta_of(w, mass)
                cell = 0.5 * beta_in * lam       # pi-mode: half a beta*lambda per cell
                beta_g = beta_in
                ta, sa = _ttf_fit(np.random.default_rng(seed * 100000 + n), beta_g)
                t, tp, sp = _ttf_eval(ta, sa, beta_in, beta_g, 0.5 * beta_g)
                # first half (phi_in = phase_ref for equal reference phases)
                phi += 0.5 * math.pi
                ph1 = phi + c * math.pi
                phase_shift = wrap_pi(phi_s - ph1)
                dw = q * e0 * cell * t * math.cos(phi_s)
                w_out = w + dw
                phi += 0.5 * math.pi
                kw = dict(length=cell, frequency=freq, cell_length_over_beta_lambda=0.5,
                          amplitude=e0, phase_ref=phi_s, phase_shift=phase_shift,
                          energy_out=w_out, beta_center=beta_g, dg=0.0, t=t, tp=tp, sp=sp,
                          fit_beta_center=beta_g, fit_beta_min=0.5 * beta_g)
                for j in range(6):
                    kw[f"fit_t{j}"] = ta[j]
                for j in range(1, 6):
                    kw[f"fit_s{j}"] = sa[j]
                elems.append(element(RFGAP_CCL, f"C{mod}T{tk:02d}G{c}", **kw))
                w = w_out
                n += 1
            bw = beta_of(w, mass)
            for j, (name, g) in enumerate((("QA", grad), ("QB", -grad))):
                elems.append(element(QUAD, f"{name}{mod}{tk:02d}", length=quad_len, gradient=g))
                phi += 2.0 * math.pi * quad_len / (lam * bw)
            elems.append(element(DRIFT, f"DT{mod}{tk:02d}", length=0.05))
            phi += 2.0 * math.pi * 0.05 / (lam * bw)
    return elems


def lattice_arrays(elems):
    """(types int32[n], params float64[n, NPARAM], names list)"""
    types = np.array([e[0] for e in elems], dtype=np.int32)
    params = np.stack([e[2] for e in elems]).astype(np.float64) if elems else np.zeros((0, NPARAM))
    names = [e[1] for e in elems]
    return types, np.ascontiguousarray(params), names
