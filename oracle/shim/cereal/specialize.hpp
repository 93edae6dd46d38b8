// Stand-in: the reference specializes this template for bit_vector; nothing reads it.
#pragma once
namespace cereal
{
enum class specialization
{
    member_serialize,
    member_load_save,
    member_load_save_minimal,
    non_member_serialize,
    non_member_load_save,
    non_member_load_save_minimal
};
template <class archive_t, class t, specialization s>
struct specialize
{};
} // namespace cereal
