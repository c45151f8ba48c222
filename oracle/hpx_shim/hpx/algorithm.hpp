// Stand-in header: the HPX algorithms used by the reference live in hpx.hpp.
// Test infrastructure only.
#pragma once
#include <hpx/hpx.hpp>
