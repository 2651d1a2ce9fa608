"""GB300-native implementation of EDEN's per-timestep simulation loop."""
