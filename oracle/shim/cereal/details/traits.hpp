// Stand-in: text-archive tag (only used for concept checks in the reference).
#pragma once
namespace cereal::traits
{
struct TextArchive
{};
} // namespace cereal::traits
