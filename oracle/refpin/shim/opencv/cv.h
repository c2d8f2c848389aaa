// Stand-in header (oracle pin, test infrastructure): the core stand-in.
#pragma once
#include "../opencv2/core/core.hpp"
