// Kernel instantiations for transform lengths 32, 80, 160, 240, 360, 480.
#include "inst.cuh"

GBN_SIZE_TU(d, GBN_L(32), GBN_L(80), GBN_L(160), GBN_L(240), GBN_L(360), GBN_L(480))
