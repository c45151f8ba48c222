// Stand-in header: hpx::execution::seq lives in hpx.hpp.
// Test infrastructure only.
#pragma once
#include <hpx/hpx.hpp>
