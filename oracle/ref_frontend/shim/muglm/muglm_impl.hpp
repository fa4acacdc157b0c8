// TEST INFRASTRUCTURE ONLY.  See muglm.hpp.
#pragma once
#include "muglm.hpp"
