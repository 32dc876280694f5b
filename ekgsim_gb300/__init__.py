"""GB300-native engine for the EkgSim simulation hot path (activation-sequence CA, Wohlfart
action potentials, dipole lead summation) behind the reference's simulator interfaces."""
