"""GB300-native vortex-lattice hot path (tinyvlm drop-in backend)."""
