"""GB300-native cyclic-symmetry modal solve (drop-in for turbomodal's tm.solve / tm.rpm_sweep path)."""
