// Minimal stand-in for boost::scoped_ptr built on std::unique_ptr.
#pragma once
#include <memory>
namespace boost {
template <class T> class scoped_ptr : public std::unique_ptr<T> {
  public:
    explicit scoped_ptr(T *p = nullptr) : std::unique_ptr<T>(p) {}
};
}
