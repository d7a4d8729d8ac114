// lie_tables.cpp -- Hall basis, bracket expansion and conversion matrices,
// built on the host once per (width, depth).
//
// The tables must equal the reference's bit for bit, so the construction
// follows the reference's published rules:
//  * Hall set (include/rpp/basis/hall_basis.hpp:35-88): key 0 is the (0,0)
//    sentinel, keys 1..W the letters (0, letter); degree d >= 2 lists pairs
//    (l, r) with deg l + deg r = d, deg l <= deg r, l < r and
//    left_parent(r) <= l, ordered by left degree, then l, then r.
//  * bracket expansion (include/rpp/basis/lie_multiplication.hpp:163-251):
//    a Hall pair maps to itself (+1), a reversed Hall pair to itself (-1), a
//    pair with r < l to minus the expansion of (r, l), otherwise the Jacobi
//    rule [l, (a, b)] = [[l, a], b] - [[l, b], a] applied recursively.
//  * t2l (include/rpp/sparse/t2l_matrix.hpp:57-142): CSC with one column per
//    tensor word (empty word included) holding the right-normed bracket
//    [w1, [w2, ..., wn]] in the Hall basis, each column of degree d >= 2
//    scaled by 1/d at the end; rows are Lie indices (key - 1).
//  * l2t (include/rpp/sparse/l2t_matrix.hpp:21-114): CSC with one column per
//    Lie index holding the commutator expansion of the Hall element, rows
//    being full tensor indices.  Digits are kept 1-based so that
//    left * W^|right| + right is the full tensor index of the concatenation.
// Coefficients are exact integers until the final 1/d scaling, so the
// summation order does not affect the result.
#include "lie_tables.hpp"

#include <algorithm>
#include <map>
#include <unordered_map>
#include <utility>

namespace rpp_gb {
namespace {

using Expansion = std::vector<std::pair<int64_t, int64_t>>;  // (key, coefficient), key-sorted

struct PairHash {
    size_t operator()(const std::pair<int64_t, int64_t>& p) const noexcept {
        return std::hash<int64_t>()(p.first * 1000003LL) ^ std::hash<int64_t>()(p.second);
    }
};

class BracketCache {
public:
    explicit BracketCache(const HallTables& h) : h_(h) {
        degree_of_.resize(static_cast<size_t>(h.true_size()));
        for (int32_t d = 0; d + 1 < static_cast<int32_t>(h.degree_begin.size()); ++d)
            for (int64_t k = h.degree_begin[d]; k < h.degree_begin[d + 1]; ++k) degree_of_[k] = d;
        for (int64_t k = 1; k < h.true_size(); ++k) key_of_[{h.pairs[2 * k], h.pairs[2 * k + 1]}] = k;
    }

    int64_t degree(int64_t key) const { return degree_of_[static_cast<size_t>(key)]; }

    int64_t find(int64_t l, int64_t r) const {
        auto it = key_of_.find({l, r});
        return it == key_of_.end() ? 0 : it->second;
    }

    const Expansion& bracket(int64_t l, int64_t r) {
        static const Expansion empty;
        if (l <= 0 || r <= 0 || l == r) return empty;
        if (l >= h_.true_size() || r >= h_.true_size()) return empty;
        if (degree(l) + degree(r) > h_.depth) return empty;
        auto it = cache_.find({l, r});
        if (it != cache_.end()) return it->second;
        Expansion res;
        if (int64_t k = find(l, r)) {
            res.emplace_back(k, 1);
        } else if (int64_t k2 = find(r, l)) {
            res.emplace_back(k2, -1);
        } else if (r < l) {
            Expansion rev = bracket(r, l);
            for (auto& e : rev) e.second = -e.second;
            res = std::move(rev);
        } else {
            std::map<int64_t, int64_t> acc;
            const int64_t a = h_.pairs[2 * r], b = h_.pairs[2 * r + 1];
            if (a > 0 && a != l) {
                const Expansion outer = bracket(l, a);
                for (const auto& [ok, ov] : outer) {
                    const Expansion inner = bracket(ok, b);
                    for (const auto& [ik, iv] : inner) acc[ik] += ov * iv;
                }
            }
            if (b != l) {
                const Expansion outer = bracket(l, b);
                for (const auto& [ok, ov] : outer) {
                    const Expansion inner = bracket(ok, a);
                    for (const auto& [ik, iv] : inner) acc[ik] -= ov * iv;
                }
            }
            for (const auto& [k, v] : acc)
                if (v != 0) res.emplace_back(k, v);
        }
        return cache_.emplace(std::make_pair(l, r), std::move(res)).first->second;
    }

private:
    const HallTables& h_;
    std::vector<int32_t> degree_of_;
    std::unordered_map<std::pair<int64_t, int64_t>, int64_t, PairHash> key_of_;
    std::unordered_map<std::pair<int64_t, int64_t>, Expansion, PairHash> cache_;
};

void append_column(CscMatrix& m, const std::map<int64_t, double>& col, double scale) {
    for (const auto& [row, v] : col) {
        if (v == 0.0) continue;
        m.indices.push_back(row);
        m.values.push_back(scale == 1.0 ? v : v * scale);
    }
    m.offsets.push_back(static_cast<int64_t>(m.indices.size()));
}

}  // namespace

HallTables build_hall_basis(int32_t width, int32_t depth) {
    HallTables h;
    h.width = width;
    h.depth = depth;
    h.degree_begin = {0, 1};
    h.pairs = {0, 0};
    if (depth > 0) {
        for (int64_t letter = 1; letter <= width; ++letter) {
            h.pairs.push_back(0);
            h.pairs.push_back(letter);
        }
        h.degree_begin.push_back(1 + width);
        for (int32_t d = 2; d <= depth; ++d) {
            for (int32_t ld = 1; 2 * ld <= d; ++ld) {
                const int32_t rd = d - ld;
                for (int64_t l = h.degree_begin[ld]; l < h.degree_begin[ld + 1]; ++l)
                    for (int64_t r = std::max(l + 1, h.degree_begin[rd]); r < h.degree_begin[rd + 1]; ++r)
                        if (h.pairs[2 * r] <= l) {
                            h.pairs.push_back(l);
                            h.pairs.push_back(r);
                        }
            }
            h.degree_begin.push_back(static_cast<int64_t>(h.pairs.size() / 2));
        }
    }
    return h;
}

CscMatrix build_conversion_matrix(const HallTables& h, int which) {
    const int64_t W = h.width;
    const int32_t D = h.depth;
    CscMatrix m;
    m.offsets.push_back(0);
    int64_t tensor_dim = 0;
    {
        int64_t p = 1;
        for (int32_t d = 0; d <= D; ++d, p *= W) tensor_dim += p;
    }
    const int64_t lie_size = (W <= 1 || D == 0) ? 0 : h.true_size() - 1;
    if (which == 0) {
        // t2l: columns = tensor words.  Column values are kept unscaled until
        // every column is built (later columns read earlier ones).
        BracketCache cache(h);
        std::vector<std::map<int64_t, double>> cols;
        cols.emplace_back();  // empty word
        if (D > 0)
            for (int64_t i = 0; i < W; ++i) cols.push_back({{i, 1.0}});
        int64_t offset = 1, prev = W;
        for (int32_t d = 2; d <= D; ++d) {
            const int64_t size = prev * W;
            for (int64_t i = 0; i < size; ++i) {
                const int64_t lparent = 1 + i / prev;
                const int64_t rparent = offset + i % prev;
                std::map<int64_t, double> frame;
                if (lparent != rparent) {
                    const double lval = cols[static_cast<size_t>(lparent)].begin()->second;
                    for (const auto& [ridx, rval] : cols[static_cast<size_t>(rparent)])
                        for (const auto& [key, c] : cache.bracket(lparent, 1 + ridx))
                            frame[key - 1] += static_cast<double>(c) * lval * rval;
                }
                for (auto it = frame.begin(); it != frame.end();)
                    it = it->second == 0.0 ? frame.erase(it) : std::next(it);
                cols.push_back(std::move(frame));
            }
            offset = 1 + offset * W;
            prev = size;
        }
        int64_t level_end = 1, level_size = 1;
        int32_t deg = 0;
        for (int64_t c = 0; c < static_cast<int64_t>(cols.size()); ++c) {
            while (c >= level_end) {
                ++deg;
                level_size *= W;
                level_end += level_size;
            }
            append_column(m, cols[static_cast<size_t>(c)], deg >= 2 ? 1.0 / static_cast<double>(deg) : 1.0);
        }
        m.outer_dim = static_cast<int64_t>(cols.size());
        m.inner_dim = lie_size;
    } else {
        // l2t: columns = Lie keys 1..true_size-1.
        std::vector<std::map<int64_t, double>> frames;
        std::vector<int32_t> degree_of(static_cast<size_t>(h.true_size()), 0);
        for (int32_t d = 0; d + 1 < static_cast<int32_t>(h.degree_begin.size()); ++d)
            for (int64_t k = h.degree_begin[d]; k < h.degree_begin[d + 1]; ++k) degree_of[k] = d;
        auto wpow = [W](int32_t e) {
            int64_t p = 1;
            for (int32_t i = 0; i < e; ++i) p *= W;
            return p;
        };
        if (D > 0)
            for (int64_t letter = 1; letter <= W; ++letter) frames.push_back({{letter, 1.0}});
        for (int32_t d = 2; d <= D; ++d) {
            for (int64_t key = h.degree_begin[d]; key < h.degree_begin[d + 1]; ++key) {
                const int64_t l = h.pairs[2 * key], r = h.pairs[2 * key + 1];
                const auto& lf = frames[static_cast<size_t>(l - 1)];
                const auto& rf = frames[static_cast<size_t>(r - 1)];
                const int64_t lo = wpow(degree_of[l]), ro = wpow(degree_of[r]);
                std::map<int64_t, double> acc;
                for (const auto& [li, lv] : lf)
                    for (const auto& [ri, rv] : rf) {
                        acc[li * ro + ri] += lv * rv;
                        acc[ri * lo + li] -= rv * lv;
                    }
                for (auto it = acc.begin(); it != acc.end();)
                    it = it->second == 0.0 ? acc.erase(it) : std::next(it);
                frames.push_back(std::move(acc));
            }
        }
        for (const auto& f : frames) append_column(m, f, 1.0);
        // The reference reports the Lie basis size (0 for width <= 1 or depth 0).
        m.outer_dim = lie_size;
        m.inner_dim = tensor_dim;
    }
    return m;
}

}  // namespace rpp_gb
