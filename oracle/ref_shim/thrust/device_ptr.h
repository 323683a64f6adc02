#pragma once
namespace thrust {
template <class T> struct device_ptr {
  T* p;
  explicit device_ptr(T* q) : p(q) {}
  device_ptr operator+(long n) const { return device_ptr(p + n); }
};
}
