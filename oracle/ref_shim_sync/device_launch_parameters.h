/* empty: the reference includes it; the shim's cuda_runtime.h declares what it would */
