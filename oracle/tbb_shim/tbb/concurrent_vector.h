// Forwarding header of the oracle-only TBB stand-in.
#pragma once
#include "../tbb_shim.h"
