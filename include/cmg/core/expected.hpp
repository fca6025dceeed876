// cmg/core/expected.hpp — value-or-error result of the C++ surface.
//
// Replaces include/cmg/core/expected.hpp of the reference for the voxelization path.
// With a C++23 library cmg::expected is std::expected. Before C++23 it is the class
// below: the subset of std::expected that callers of voxelize use (has_value, bool
// conversion, value, error, dereference, value_or, construction from a value or from
// cmg::unexpected). Its storage is a std::variant<T, E>, the layout the reference's
// own pre-C++23 form has, so results cross between code built against either header
// unchanged. Build the library and its callers with the same -std (libcmg_c.so's C++
// surface is built with -std=c++20).
#pragma once

#include <utility>

#if defined(__cpp_lib_expected) && __cpp_lib_expected >= 202202L
#include <expected>

namespace cmg {
template <class T, class E>
using expected = std::expected<T, E>;
template <class E>
using unexpected = std::unexpected<E>;
}  // namespace cmg

#else
#include <variant>

namespace cmg {

// The error alternative, tagged so that it cannot be mistaken for a value.
template <class E>
class unexpected {
public:
    explicit unexpected(E err) : err_(std::move(err)) {}
    E& error() & noexcept { return err_; }
    const E& error() const& noexcept { return err_; }
    E&& error() && noexcept { return std::move(err_); }

private:
    E err_;
};

template <class T, class E>
class expected {
    static constexpr std::size_t kValue = 0, kError = 1;

public:
    using value_type = T;
    using error_type = E;

    expected() : v_(std::in_place_index<kValue>) {}
    expected(const T& value) : v_(std::in_place_index<kValue>, value) {}
    expected(T&& value) : v_(std::in_place_index<kValue>, std::move(value)) {}
    expected(const unexpected<E>& e) : v_(std::in_place_index<kError>, e.error()) {}
    expected(unexpected<E>&& e) : v_(std::in_place_index<kError>, std::move(e).error()) {}

    bool has_value() const noexcept { return v_.index() == kValue; }
    explicit operator bool() const noexcept { return has_value(); }

    T& value() & { return std::get<kValue>(v_); }
    const T& value() const& { return std::get<kValue>(v_); }
    T&& value() && { return std::move(std::get<kValue>(v_)); }
    E& error() & { return std::get<kError>(v_); }
    const E& error() const& { return std::get<kError>(v_); }
    E&& error() && { return std::move(std::get<kError>(v_)); }

    T& operator*() & noexcept { return *std::get_if<kValue>(&v_); }
    const T& operator*() const& noexcept { return *std::get_if<kValue>(&v_); }
    T* operator->() noexcept { return std::get_if<kValue>(&v_); }
    const T* operator->() const noexcept { return std::get_if<kValue>(&v_); }

    template <class U>
    T value_or(U&& other) const& {
        if (has_value()) return value();
        return static_cast<T>(std::forward<U>(other));
    }

private:
    std::variant<T, E> v_;
};

}  // namespace cmg
#endif
