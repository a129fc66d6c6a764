"""GB300-native beam-lattice energy/gradient + L-BFGS path (see include/mcg.h)."""
