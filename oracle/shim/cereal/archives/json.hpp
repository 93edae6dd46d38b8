// Stand-in: JSON archives accept and discard everything, so config::read_from/write_to are no-ops in the oracle build.
#pragma once
#include <iosfwd>
#include <cereal/cereal.hpp>
namespace cereal
{
class JSONInputArchive : public detail::InputArchiveBase, public traits::TextArchive
{
public:
    explicit JSONInputArchive(std::istream &)
    {}
    template <class... ts>
    void operator()(ts &&...)
    {}
};
class JSONOutputArchive : public detail::OutputArchiveBase, public traits::TextArchive
{
public:
    explicit JSONOutputArchive(std::ostream &)
    {}
    template <class... ts>
    void operator()(ts &&...)
    {}
};
} // namespace cereal
