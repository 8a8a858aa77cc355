"""GB300-native NNAP energy/force/virial evaluation."""
