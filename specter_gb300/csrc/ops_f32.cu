// FP32 instantiation of the host operations (ops_impl.cuh).
#include "ops_impl.cuh"
