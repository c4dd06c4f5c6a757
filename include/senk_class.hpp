/**
 * @file senk_class.hpp
 * @brief senk::sparse::SpVec, the growable sparse row of the SenK API (drop-in
 *        for include/senk_class.hpp:23-123): parallel arrays of value, level and
 *        index, appended in order.
 */
#ifndef SENK_CLASS_HPP
#define SENK_CLASS_HPP

#include <tuple>
#include <vector>

namespace senk {
namespace sparse {

template <typename T1, typename T2>
class SpVec {
public:
    SpVec() { reserve(8); }
    /** Append one entry. */
    inline void Append(T1 v, T2 lev, int idx)
    {
        val_.push_back(v);
        lev_.push_back(lev);
        idx_.push_back(idx);
    }
    /** Append t_len entries from parallel arrays. */
    inline void Append(T1 *v, T2 *lev, int *idx, int t_len)
    {
        val_.insert(val_.end(), v, v + t_len);
        lev_.insert(lev_.end(), lev, lev + t_len);
        idx_.insert(idx_.end(), idx, idx + t_len);
    }
    inline int GetLen() { return (int)idx_.size(); }
    inline T1 GetVal(int i) { return val_[i]; }
    inline T2 GetLev(int i) { return lev_[i]; }
    inline int GetIdx(int i) { return idx_[i]; }
    inline std::tuple<T1, T2, int> Get(int i) { return {val_[i], lev_[i], idx_[i]}; }
    inline void Clear()
    {
        val_.clear();
        lev_.clear();
        idx_.clear();
    }

private:
    void reserve(size_t n)
    {
        val_.reserve(n);
        lev_.reserve(n);
        idx_.reserve(n);
    }
    std::vector<T1> val_;
    std::vector<T2> lev_;
    std::vector<int> idx_;
};

}  // namespace sparse
}  // namespace senk

#endif
