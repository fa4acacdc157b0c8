#pragma once
#include "intrusive_hash_map.hpp"
