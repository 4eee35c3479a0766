"""Physical constants and ids, identical to the reference's src/constants.f90."""
import math

# src/constants.f90:30-39
SQRT2 = math.sqrt(2.0)
SQRT3 = math.sqrt(3.0)
PI = math.acos(-1.0)
KB = 8.61733238496e-5          # eV / K
HBAR = 0.6582119514467406      # eV fs
TWELFTH = 1.0 / 12.0
TOLERANCE = 1.0e-9             # constants.f90:94

# src/constants.f90:157-170
AMU2MASS = 103.638239276       # amu -> eV fs^2 / A^2
DEG2RAD = PI / 180.0
BOHR2ANG = 0.529177211
ANG2BOHR = 1.0 / BOHR2ANG
HA2EV = 27.21138602
HABOHR2EVANG = HA2EV * ANG2BOHR

# src/constants.f90:64-71
PES_ID_LJ = 2001
PES_ID_EMT = 2003
PES_ID_NENE = 2008
PES_ID_NO_INTERACTION = 2007

# src/constants.f90:107-115
PROP_ID_VERLET = 1001
PROP_ID_LANGEVIN = 1003
PROP_ID_ANDERSEN = 1005
PROP_ID_PILE = 1006
PROP_ID_LANGEVIN_CONST = 1007   # constant friction: this engine's addition
ENERGY_AND_FORCE = 3001
ENERGY_ONLY = 3002

PROP_KEYWORDS = {"ver": PROP_ID_VERLET, "lan": PROP_ID_LANGEVIN, "and": PROP_ID_ANDERSEN,
                 "pil": PROP_ID_PILE, "lac": PROP_ID_LANGEVIN_CONST}

# element masses used by the synthetic workloads (amu)
MASS_AMU = {"H": 1.008, "D": 2.014, "C": 12.011, "Au": 196.967, "Pt": 195.084}
