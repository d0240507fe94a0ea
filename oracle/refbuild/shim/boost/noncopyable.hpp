// Declaration-only stand-in for boost::noncopyable, so the reference
// ray-tracer sources compile without Boost installed.
#pragma once
namespace boost {
class noncopyable {
  protected:
    noncopyable() = default;
    ~noncopyable() = default;
    noncopyable(const noncopyable &) = delete;
    noncopyable &operator=(const noncopyable &) = delete;
};
}
