// A minimal owning pointer map with boost::ptr_map's interface as the
// reference uses it (insert of a raw pointer, at, count, iteration yielding
// (key, pointer) pairs), for the cross-check build.  Not Boost code.
#pragma once
#include <map>
#include <memory>
#include <stdexcept>
#include <utility>

namespace boost {

template <class K, class T>
class ptr_map {
    std::map<K, std::unique_ptr<T>> m_;
    mutable std::map<K, T*> view_;

  public:
    std::pair<typename std::map<K, T*>::iterator, bool> insert(const K& k, T* p) {
        auto r = m_.emplace(k, std::unique_ptr<T>(p));
        if (!r.second) delete p;
        view_[k] = r.first->second.get();
        return {view_.find(k), r.second};
    }
    T& at(const K& k) { auto it = m_.find(k); if (it == m_.end()) throw std::out_of_range("ptr_map"); return *it->second; }
    const T& at(const K& k) const { auto it = m_.find(k); if (it == m_.end()) throw std::out_of_range("ptr_map"); return *it->second; }
    std::size_t count(const K& k) const { return m_.count(k); }
    std::size_t size() const { return m_.size(); }
    typename std::map<K, T*>::const_iterator begin() const { return view_.begin(); }
    typename std::map<K, T*>::const_iterator end() const { return view_.end(); }
    void erase(const K& k) { view_.erase(k); m_.erase(k); }
};

}  // namespace boost
