// freelist.cpp - see freelist.h.
#include "freelist.h"

namespace vrt {

void FreeList::grow(uint32_t new_capacity) {
    if (new_capacity <= capacity_) return;
    uint32_t start = capacity_ + 1, len = new_capacity - capacity_;
    capacity_ = new_capacity;
    // coalesce with a free range that ends at the old capacity
    if (!ranges_.empty()) {
        auto last = std::prev(ranges_.end());
        if (last->first + last->second == start) {
            last->second += len;
            return;
        }
    }
    ranges_[start] = len;
}

void FreeList::take_front(std::map<uint32_t, uint32_t>::iterator it, uint32_t count) {
    uint32_t start = it->first, len = it->second;
    ranges_.erase(it);
    if (len > count) ranges_[start + count] = len - count;
    allocated_ += count;
}

void FreeList::take_exact(uint32_t start, uint32_t count) {
    if (count == 0) return;
    auto it = ranges_.upper_bound(start);
    --it;  // range containing start
    uint32_t rs = it->first, rl = it->second;
    ranges_.erase(it);
    if (start > rs) ranges_[rs] = start - rs;
    uint32_t end = start + count, rend = rs + rl;
    if (rend > end) ranges_[end] = rend - end;
    allocated_ += count;
}

uint32_t FreeList::realloc(uint32_t base, uint32_t cur, uint32_t want) {
    if (want <= cur && base != 0) return base;
    if (base != 0) {
        // grow in place into the free range that starts right at the end
        auto it = ranges_.find(base + cur);
        if (it != ranges_.end() && base + want < it->first + it->second) {
            take_front(it, base + want - it->first);
            return base;
        }
        free(base, cur);
    }
    auto best = ranges_.end();
    for (auto it = ranges_.begin(); it != ranges_.end(); ++it)
        if (it->second >= want && (best == ranges_.end() || it->second < best->second)) best = it;
    if (best == ranges_.end()) {
        if (base != 0) take_exact(base, cur);  // restore the old allocation
        return 0;
    }
    uint32_t start = best->first;
    take_front(best, want);
    return start;
}

void FreeList::free(uint32_t base, uint32_t size) {
    if (size == 0) return;
    allocated_ -= size;
    auto it = ranges_.emplace(base, size).first;
    auto next = std::next(it);
    if (next != ranges_.end() && it->first + it->second == next->first) {
        it->second += next->second;
        ranges_.erase(next);
    }
    if (it != ranges_.begin()) {
        auto prev = std::prev(it);
        if (prev->first + prev->second == it->first) {
            prev->second += it->second;
            ranges_.erase(it);
        }
    }
}

uint32_t FreeList::high_water() const {
    // the end of the allocation that reaches furthest: capacity+1 unless the last
    // free range runs to the end
    if (ranges_.empty()) return capacity_ + 1;
    auto last = std::prev(ranges_.end());
    if (last->first + last->second == capacity_ + 1) return last->first;
    return capacity_ + 1;
}

void FreeList::assign_used(uint32_t capacity, const std::vector<std::pair<uint32_t, uint32_t>>& used) {
    ranges_.clear();
    capacity_ = capacity;
    allocated_ = 0;
    uint32_t next = 1;  // first slot not yet accounted for
    for (const auto& u : used) {
        if (u.second == 0) continue;
        if (u.first > next) ranges_[next] = u.first - next;
        allocated_ += u.second;
        next = u.first + u.second;
    }
    if (next <= capacity) ranges_[next] = capacity + 1 - next;
}

bool sector_free(FreeList& fl, SectorSlots& s, uint64_t remove) {
    uint64_t nm = s.mask & ~remove;
    if (nm == s.mask) return true;
    uint32_t cur = (uint32_t)__builtin_popcountll(s.mask);
    uint32_t nsz = (uint32_t)__builtin_popcountll(nm);
    fl.free(s.base + nsz, cur - nsz);
    if (nm == 0) s.base = 0;
    s.mask = nm;
    return true;
}

bool sector_alloc(FreeList& fl, SectorSlots& s, uint64_t add) {
    uint64_t nm = s.mask | add;
    if (nm == s.mask) return true;
    uint32_t cur = (uint32_t)__builtin_popcountll(s.mask);
    uint32_t nsz = (uint32_t)__builtin_popcountll(nm);
    uint32_t nb = fl.realloc(s.base, cur, nsz);
    if (nb == 0) return false;
    s.base = nb;
    s.mask = nm;
    return true;
}

}  // namespace vrt
