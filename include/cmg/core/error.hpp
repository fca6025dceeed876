// cmg/core/error.hpp — recoverable failures of the C++ surface.
//
// Replaces include/cmg/core/error.hpp of the reference (:39-56) for the voxelization
// path: a bad input comes back as a MeshError value inside cmg::expected, never as an
// exception. The codes are the reference's, in its order (they map one to one onto
// the C ABI's cmg_status values 1-6).
#pragma once

#include <cstddef>
#include <stdexcept>
#include <string>
#include <utility>

namespace cmg {

// Misuse and broken invariants (not returned by voxelize).
class error : public std::runtime_error {
public:
    explicit error(const std::string& what) : std::runtime_error(what) {}
};

enum class MeshErrorCode {
    InvalidInput,
    SelfIntersection,
    UnsupportedOption,
    QualityNotMet,
    NotImplemented,
    Internal,
};

struct MeshError {
    MeshErrorCode code = MeshErrorCode::Internal;
    std::string message;

    MeshError() = default;
    MeshError(MeshErrorCode c, std::string msg) : code(c), message(std::move(msg)) {}
};

struct ParseError {
    std::string message;
    std::size_t position = 0;

    ParseError() = default;
    explicit ParseError(std::string msg, std::size_t pos = 0) : message(std::move(msg)), position(pos) {}
};

}  // namespace cmg
