// Forwarding header: OpenCLIPER GroupwiseRegistration process on the GB300 library.
#pragma once
#include "../gbn_facade.hpp"
