// Forwarding header: OpenCLIPER ComplexAbs process on the GB300 library.
#pragma once
#include "../gbn_facade.hpp"
