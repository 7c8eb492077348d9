// Forwarding header: OpenCLIPER VectorNormalization process on the GB300 library.
#pragma once
#include "../../gbn_facade.hpp"
