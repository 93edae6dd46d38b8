// Stand-in: base_class<B>(derived*) wrapper holding the base object, for archives that serialise it (the byte
// archive of oracle/ref_driver.cpp); the reference only constructs it and passes it to its archive.
#pragma once
namespace cereal
{
template <class base_t>
struct base_class
{
    base_t * base_ptr;
    template <class derived_t>
    base_class(derived_t const * d) : base_ptr{const_cast<base_t *>(static_cast<base_t const *>(d))}
    {}
};
} // namespace cereal
