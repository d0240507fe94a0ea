// Minimal stand-in for boost::shared_array built on std::shared_ptr<T[]>.
#pragma once
#include <memory>
#include <cstddef>
namespace boost {
template <class T> class shared_array {
  public:
    shared_array() = default;
    explicit shared_array(T *p) : _p(p, [](T *q) { delete[] q; }) {}
    T &operator[](std::ptrdiff_t i) const { return _p.get()[i]; }
    T *get() const { return _p.get(); }
    void reset(T *p = nullptr) { _p.reset(p, [](T *q) { delete[] q; }); }
    explicit operator bool() const { return static_cast<bool>(_p); }
  private:
    std::shared_ptr<T> _p;
};
}
