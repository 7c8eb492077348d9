// Kernel instantiations for transform lengths 40, 96, 168, 256, 384, 504.
#include "inst.cuh"

GBN_SIZE_TU(e, GBN_L(40), GBN_L(96), GBN_L(168), GBN_L(256), GBN_L(384), GBN_L(504))
