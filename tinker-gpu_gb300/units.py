"""Physical constants in Tinker units (Tinker units.f, as used through
ext/interface/cpp/tinker/detail/units.hh by the reference)."""

BOHR = 0.529177210903  # Angstrom per bohr
DEBYE = 4.8033324  # Debye per e*Angstrom
ELECTRIC = 332.0637133  # kcal*Angstrom/(mol*e^2), Coulomb constant
