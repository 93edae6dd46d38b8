// Stand-in: base_class<B>(derived*) wrapper; never archived.
#pragma once
namespace cereal
{
template <class base_t>
struct base_class
{
    template <class derived_t>
    base_class(derived_t const *)
    {}
};
} // namespace cereal
