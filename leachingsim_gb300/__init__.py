"""GB300-native LeachingSim hot path: CUDA kernels behind a C-ABI (include/leachingsim.h)."""
