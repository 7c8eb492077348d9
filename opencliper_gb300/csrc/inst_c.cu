// Kernel instantiations for transform lengths 24, 72, 144, 224, 336, 448.
#include "inst.cuh"

GBN_SIZE_TU(c, GBN_L(24), GBN_L(72), GBN_L(144), GBN_L(224), GBN_L(336), GBN_L(448))
