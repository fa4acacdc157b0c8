// Stand-in for Granite's Util containers: declarations only, never instantiated.
#pragma once
#include <stdint.h>
#include "muglm/muglm_impl.hpp"
namespace Util
{
using Hash = uint64_t;
template <typename T> struct IntrusiveHashMapEnabled {};
template <typename T, typename D = void> struct IntrusivePtrEnabled {};
template <typename T> struct IntrusivePtr {};
template <typename T> struct ObjectPool {};
template <typename T> struct IntrusiveHashMapHolder {};
template <typename T> struct IntrusiveHashMap {};
}
