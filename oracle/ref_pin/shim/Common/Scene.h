// Stand-in for glim::Model (VoxelMap.h only declares a function taking it).
#pragma once
#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <string_view>
#include <unordered_map>
#include <vector>
#include <cassert>
#include <stdexcept>
#include <bit>
namespace glim {
struct Model;
}
