// Test infrastructure only (oracle build of the reference). Minimal stand-in
// for boost::alignment::aligned_allocator<T, Alignment>, the one boost header
// the reference's math code uses (Math/Color.h). Backed by C++17 aligned new.
#pragma once
#include <cstddef>
#include <new>

namespace boost { namespace alignment {

template <class T, std::size_t Alignment = alignof(T)>
class aligned_allocator
{
public:
    using value_type = T;
    template <class U> struct rebind { using other = aligned_allocator<U, Alignment>; };

    aligned_allocator() noexcept = default;
    template <class U> aligned_allocator(const aligned_allocator<U, Alignment>&) noexcept {}

    T* allocate(std::size_t n)
    {
        return static_cast<T*>(::operator new(n * sizeof(T), std::align_val_t(Alignment)));
    }
    void deallocate(T* p, std::size_t) noexcept
    {
        ::operator delete(p, std::align_val_t(Alignment));
    }
    template <class U> bool operator==(const aligned_allocator<U, Alignment>&) const noexcept { return true; }
    template <class U> bool operator!=(const aligned_allocator<U, Alignment>&) const noexcept { return false; }
};

} }
