// Kernel instantiations for transform lengths 16, 64, 128, 216, 320, 432.
#include "inst.cuh"

GBN_SIZE_TU(b, GBN_L(16), GBN_L(64), GBN_L(128), GBN_L(216), GBN_L(320), GBN_L(432))
