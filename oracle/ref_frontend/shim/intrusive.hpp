// TEST INFRASTRUCTURE ONLY.  Stand-in for the Granite header of this name.
#pragma once
#include "granite_shim.hpp"
