// TEST INFRASTRUCTURE ONLY.  Stand-in for Granite's Vulkan image types: the
// recording renderer hands out empty, reference-counted image handles.
#pragma once
#include "device.hpp"
