// TEST INFRASTRUCTURE ONLY.  Stand-in for Granite's Vulkan device header.  No
// Vulkan is used: the reference's GSRenderer is replaced by a recording
// implementation, and these are the plain handle and value types its header
// names as members and parameters, so that the CPU frontend compiles.
#pragma once
#include "granite_shim.hpp"
#include <stdint.h>

typedef uint64_t VkDeviceSize;
typedef uint64_t VkDeviceAddress;
struct VkOffset2D { int32_t x, y; };
struct VkExtent2D { uint32_t width, height; };
struct VkRect2D { VkOffset2D offset; VkExtent2D extent; };
struct VkImageMemoryBarrier2 { uint32_t unused; };
struct VkBufferMemoryBarrier2 { uint32_t unused; };
typedef uint32_t VkFormat;
typedef uint32_t VkImageLayout;
typedef uint64_t VkPipelineStageFlags2;
typedef uint64_t VkAccessFlags2;

namespace Vulkan
{
// Limits as the frontend's table sizes use them (Granite's limits.hpp).
static constexpr unsigned VULKAN_MAX_UBO_SIZE = 64 * 1024;
static constexpr unsigned VULKAN_NUM_BINDINGS_BINDLESS_VARYING = 16 * 1024;

class Device;
class Program;
class Shader;
class Image;
// The recording renderer's images only carry their extent.
struct ImageView
{
	const Image *image = nullptr;
	uint32_t width = 0, height = 0;
	uint32_t get_view_width() const { return width; }
	uint32_t get_view_height() const { return height; }
	const Image &get_image() const { return *image; }
};
struct ImageCreateInfo
{
	uint32_t width = 0, height = 0, levels = 1;
};
class Image : public Util::IntrusivePtrEnabled<Image>
{
public:
	Image(uint32_t w = 0, uint32_t h = 0, uint32_t levels = 1) : width(w), height(h)
	{
		view.image = this;
		view.width = w;
		view.height = h;
		info.width = w;
		info.height = h;
		info.levels = levels;
	}
	const ImageCreateInfo &get_create_info() const { return info; }
	ImageCreateInfo info;
	const ImageView &get_view() const { return view; }
	uint32_t get_width(uint32_t = 0) const { return width; }
	uint32_t get_height(uint32_t = 0) const { return height; }
	uint32_t width, height;
	ImageView view;
};
using ImageHandle = Util::IntrusivePtr<Image>;
class Buffer : public Util::IntrusivePtrEnabled<Buffer> {};
using BufferHandle = Util::IntrusivePtr<Buffer>;
class BufferView : public Util::IntrusivePtrEnabled<BufferView> {};
using BufferViewHandle = Util::IntrusivePtr<BufferView>;
class CommandBuffer : public Util::IntrusivePtrEnabled<CommandBuffer>
{
public:
	enum class Type { Generic, AsyncGraphics, AsyncCompute, AsyncTransfer };
};
using CommandBufferHandle = Util::IntrusivePtr<CommandBuffer>;
class SemaphoreHolder : public Util::IntrusivePtrEnabled<SemaphoreHolder> {};
using Semaphore = Util::IntrusivePtr<SemaphoreHolder>;
class QueryPoolResult : public Util::IntrusivePtrEnabled<QueryPoolResult> {};
using QueryPoolHandle = Util::IntrusivePtr<QueryPoolResult>;
class BindlessDescriptorPool : public Util::IntrusivePtrEnabled<BindlessDescriptorPool> {};
using BindlessDescriptorPoolHandle = Util::IntrusivePtr<BindlessDescriptorPool>;
struct BufferBlockAllocation { uint8_t *host = nullptr; VkDeviceSize offset = 0; };
}
