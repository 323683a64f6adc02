#pragma once
#include "device_ptr.h"
namespace thrust {
template <class T, class V> void fill(device_ptr<T> a, device_ptr<T> b, V v) { for (T* p = a.p; p != b.p; ++p) *p = (T)v; }
}
