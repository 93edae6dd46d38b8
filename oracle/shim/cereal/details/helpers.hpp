// Stand-in: archive base classes (only used for concept checks in the reference).
#pragma once
namespace cereal::detail
{
struct OutputArchiveBase
{};
struct InputArchiveBase
{};
} // namespace cereal::detail
