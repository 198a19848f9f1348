"""Python mirror of the flat system layout of ``include/posidonius_gb300.h``.

One system = ``sys_i64[SI_COUNT]`` + ``sys_f64[SF_COUNT]`` + ``nmax`` bodies of
``body_i64[BI_COUNT]`` and ``body_f64[BF_COUNT]`` (row-major, bodies in the
reference's particle order).  ``tests/test_layout.py`` checks every constant
here against the C header.
"""

# posi_status
OK = 0
COMPLETED = 1
ERR_ARG = -1
ERR_IO = -2
ERR_PARSE = -3
ERR_UNSUPPORTED = -4
ERR_CUDA = -5
ERR_PHYSICS = -6
ERR_STATE = -7

# posi_system_status
SYS_OK = 0
SYS_ROCHE = 1
SYS_COLLISION = 2
SYS_EJECTED = 3
SYS_ZERO_INERTIA = 4
SYS_BISECTION_LIMIT = 5
SYS_COMPLETED = 6
SYS_FATAL_MASK = 0xFF
SYS_WARN_NONCONVERGED = 1 << 8
SYS_WARN_TIMESTEP = 1 << 9

# posi_coords
JACOBI = 0
DEMOCRATIC_HELIOCENTRIC = 1
WHDS = 2

# posi_effect_kind
EFFECT_DISABLED = 0
EFFECT_CENTRAL = 1
EFFECT_ORBITING = 2

# posi_gr_impl
GR_KIDDER1995 = 0
GR_ANDERSON1975 = 1
GR_NEWHALL1983 = 2

# posi_evolution
EVO_NON_EVOLVING = 0
EVO_LECONTE2011 = 1
EVO_BARAFFE1998 = 2
EVO_BARAFFE2015 = 3
EVO_LECONTE_CHABRIER2013 = 4

# posi_sys_i64_field
(SI_N, SI_HOST, SI_COORDS, SI_TIDES, SI_FLAT, SI_GR, SI_EVOLUTION, SI_ITERATION, SI_N_HIST,
 SI_TIMESTEP_WARNING, SI_STATUS, SI_FAIL_STEP, SI_FAIL_PAIR, SI_LAST_MIDPOINT_ITERS, SI_GR_IMPL, SI_WIND,
 SI_COUNT) = range(17)

# posi_sys_f64_field
(SF_DT, SF_HALF_DT, SF_TIME, SF_TIME_LIMIT, SF_LAST_HIST, SF_HIST_PERIOD, SF_LAST_REC, SF_REC_PERIOD,
 SF_INITIAL_TIME, SF_COUNT) = range(10)

# posi_body_i64_field
(BI_TIDES_KIND, BI_FLAT_KIND, BI_GR_KIND, BI_EVO_TYPE, BI_EVO_OFFSET, BI_EVO_LEN, BI_EVO_LEFT, BI_WIND_KIND,
 BI_COUNT) = range(9)

# posi_body_f64_field
(BF_MASS, BF_MASS_G, BF_RADIUS, BF_RG2, BF_MOI,
 BF_PX, BF_PY, BF_PZ, BF_VX, BF_VY, BF_VZ, BF_AX, BF_AY, BF_AZ,
 BF_LX, BF_LY, BF_LZ, BF_SX, BF_SY, BF_SZ, BF_NSV2,
 BF_EVX, BF_EVY, BF_EVZ, BF_ELX, BF_ELY, BF_ELZ,
 BF_SIGMA, BF_K2, BF_K2F,
 BF_ADDAX, BF_ADDAY, BF_ADDAZ, BF_DLX, BF_DLY, BF_DLZ,
 BF_DENERGY_DT, BF_LAG_ANGLE,
 BF_TD_DIST, BF_TD_VR, BF_TD_ORTHO, BF_TD_DPM, BF_TD_PX, BF_TD_PY, BF_TD_PZ, BF_TD_VX, BF_TD_VY, BF_TD_VZ,
 BF_TD_LX, BF_TD_LY, BF_TD_LZ, BF_WIND_K, BF_WIND_RSAT, BF_WIND_RSAT2, BF_COUNT) = range(55)

MAX_BODIES = 32

# posi_mode
MODE_EXACT = 0
MODE_FAST = 1

# posi_mapping
MAP_AUTO = 0
MAP_THREAD = 1
MAP_LANES2 = 2
MAP_LANES4 = 4
MAP_LANES8 = 8
MAP_LANES16 = 16
MAP_WARP = 32

POS = slice(BF_PX, BF_PZ + 1)
VEL = slice(BF_VX, BF_VZ + 1)
ACC = slice(BF_AX, BF_AZ + 1)
ANG = slice(BF_LX, BF_LZ + 1)
SPIN = slice(BF_SX, BF_SZ + 1)

# posi_adjoint_flag
ADJ_KEPLER = 1
ADJ_ZERO_INERTIA = 2
ADJ_FROZEN = 4
ADJ_UNSUPPORTED = 8

# posi_seed_param (parameters a tangent direction of the many-body engine perturbs)
SEED_SIGMA = 0
SEED_K2 = 1
