// Shared host-side definitions for the femocs_gb300 library.
#pragma once

#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>
#include <stdexcept>

namespace fgb {

// Cell/node classification codes, numerically identical to the reference's TYPES
// (include/Globals.h:37-56) because they appear in exported marker arrays.
enum : int {
    kBulk = 1,
    kSurface = 2,
    kVacuum = 3,
    kTetNode = 1,
    kEdgeCentroid = 2,
    kFaceCentroid = 3,
    kTetCentroid = 4,
};

// Boundary ids of the vacuum hex mesh, as in the reference (include/Globals.h BoundaryID).
enum : int {
    kBidCopper = 2,
    kBidSides = 4,
    kBidTop = 8,
};

struct Error : std::runtime_error {
    explicit Error(const std::string& m) : std::runtime_error(m) {}
};

#define FGB_REQUIRE(cond, msg)                                                  \
    do {                                                                        \
        if (!(cond)) throw ::fgb::Error(std::string(__FILE__) + ":" +           \
                                        std::to_string(__LINE__) + ": " + (msg)); \
    } while (0)

// Last error message of the calling thread, exposed through the C ABI.
void set_last_error(const std::string& msg);
const char* last_error();

}  // namespace fgb
