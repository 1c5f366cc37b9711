"""GB300-native SKID group-finding hot path (see include/skid_gpu.h for the C ABI)."""
