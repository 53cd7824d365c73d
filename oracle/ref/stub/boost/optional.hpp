#pragma once
#include <optional>
namespace boost { template <class T> using optional = std::optional<T>; }
