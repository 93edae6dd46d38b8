// Stand-in for cereal/cereal.hpp: name-value pairs and binary blobs collapse to no-ops.
#pragma once
#include <cstddef>
#include <cereal/access.hpp>
#include <cereal/details/helpers.hpp>
#include <cereal/details/traits.hpp>
#include <cereal/macros.hpp>
#include <cereal/specialize.hpp>
namespace cereal
{
template <class t>
t & make_nvp(char const *, t & value)
{
    return value;
}
template <class t>
t const & make_nvp(char const *, t const & value)
{
    return value;
}
struct binary_data_t
{
    void const * ptr;
    std::size_t size;
};
inline binary_data_t binary_data(void const * ptr, std::size_t size)
{
    return {ptr, size};
}
} // namespace cereal
