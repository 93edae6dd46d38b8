// Stand-in: cereal::access is only befriended by the reference.
#pragma once
namespace cereal
{
class access
{};
} // namespace cereal
