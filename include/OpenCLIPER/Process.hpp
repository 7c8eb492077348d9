// Forwarding header: OpenCLIPER Process API on the GB300 library.
#pragma once
#include "gbn_facade.hpp"
