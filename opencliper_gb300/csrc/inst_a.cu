// Kernel instantiations for transform lengths 8, 56, 120, 200, 288, 400.
#include "inst.cuh"

GBN_SIZE_TU(a, GBN_L(8), GBN_L(56), GBN_L(120), GBN_L(200), GBN_L(288), GBN_L(400))
