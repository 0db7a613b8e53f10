/* empty: launch parameters come from cuda_runtime.h in the CPU shim */
