"""Physical constants of the reference's internal unit system (angstrom, dalton, picosecond).

The reference parses quantities such as ``0.3729 eV`` through its onika unit
layer, which is not part of the exaNBody tree. The two constants below are the
ones that reproduce the reference's own golden data
(contribs/microStamp/samples/benchmark_lj_snap/check_values_lj_Ni.dat) to
1e-9 in acceleration; the values quoted by later CODATA releases leave a
7.9e-6 relative bias in eps/m that the golden check rejects.
"""

ELEMENTARY_CHARGE_J = 1.6021892e-19  # joule per electron-volt
DALTON_KG = 1.66053904e-27  # kilogram per dalton

# energy unit of the internal system: Da * angstrom^2 / ps^2, in joule
_INTERNAL_ENERGY_J = DALTON_KG * 1e-20 / 1e-24


def ev_to_internal(x_ev):
    """Convert an energy in eV to Da*angstrom^2/ps^2."""
    return x_ev * ELEMENTARY_CHARGE_J / _INTERNAL_ENERGY_J
