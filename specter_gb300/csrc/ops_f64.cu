// FP64 instantiation of the host operations (ops_impl.cuh).
#define SG_PREC_DOUBLE
#include "ops_impl.cuh"
