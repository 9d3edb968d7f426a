// Internal helpers of the C++ API implementation.
#pragma once

namespace qtnh {
namespace detail {
/// Maps a C ABI status to the reference's exception types.
void check(int rc);
}
}
