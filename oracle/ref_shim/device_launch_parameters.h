/* empty: see cuda_runtime.h */
