// Stand-in header: the names live in pvfmm_common.hpp.
// TEST INFRASTRUCTURE ONLY (oracle/_ref).
#pragma once
#include <pvfmm_common.hpp>
