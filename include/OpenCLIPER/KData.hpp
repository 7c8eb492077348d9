// Forwarding header: OpenCLIPER KData API on the GB300 library.
#pragma once
#include "gbn_facade.hpp"
