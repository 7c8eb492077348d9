// Forwarding header: OpenCLIPER ComplexAbsPow2 process on the GB300 library.
#pragma once
#include "../gbn_facade.hpp"
