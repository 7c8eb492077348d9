// Kernel instantiations for transform lengths 48, 112, 192, 280, 392, 512.
#include "inst.cuh"

GBN_SIZE_TU(f, GBN_L(48), GBN_L(112), GBN_L(192), GBN_L(280), GBN_L(392), GBN_L(512))
