// Stand-in for boost::scoped_ptr: a unique_ptr has the same ownership semantics for its one use.
#pragma once
#include <memory>
namespace boost { template <class T> using scoped_ptr = std::unique_ptr<T>; }
