#pragma once
#include <stdint.h>
namespace Vulkan { struct ImageHandle {}; }
typedef uint64_t VkDeviceAddress;
