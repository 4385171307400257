// Build shim for compiling the unmodified LIFE reference sources without Boost.
// The reference uses only exists / remove / remove_all / rename /
// create_directory / directory_iterator / path, all of which std::filesystem
// provides with the same names. The reference also relies on Boost pulling in
// these standard headers transitively.
#pragma once
#include <array>
#include <vector>
#include <fstream>
#include <string>
#include <limits>
#include <algorithm>
#include <cstdint>
#include <filesystem>
namespace boost { namespace filesystem = std::filesystem; }
