/* A minimal stand-in for nlohmann/json (https://github.com/nlohmann/json,
 * which the reference includes as <json.hpp> but does not vendor), written
 * for building the reference's glTF loader (src/data/gltf.cpp) as a test
 * oracle.  TEST INFRASTRUCTURE ONLY: nothing in the product includes it.
 *
 * It covers the calls that loader makes, with nlohmann's documented
 * semantics:
 *   - parse(first, last) of RFC 8259 text; a number without fraction or
 *     exponent is an integer (signed when it starts with '-', else
 *     unsigned), any other number a double from strtod;
 *   - operator[] by key (the non-const form inserts a null member when the
 *     key is absent, the const form of an absent key yields null) and by
 *     index; contains(); size() (0 for null, 1 for a scalar);
 *   - get<T>() of a number as static_cast<T>(stored value), of a string as
 *     std::string, of a boolean;
 *   - value(key, default): the member converted to the default's type (a
 *     std::string for a const char * default), or the default when absent;
 *   - implicit conversion to std::string, comparison with a C string;
 *   - range-for over an array's elements (or an object's values).
 */
#pragma once

#include <cerrno>
#include <cstdint>
#include <cstdlib>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

namespace nlohmann {

class json {
public:
    enum class kind { null, boolean, integer, unsigned_integer, floating, string, array, object };

    json() = default;

    template <class It> static json parse(It first, It last)
    {
        std::string text(first, last);
        size_t at = 0;
        json j = parse_value(text, at);
        skip_ws(text, at);
        if (at != text.size())
            throw std::runtime_error("json: trailing characters");
        return j;
    }

    // ------------------------------------------------------------ access --
    json &operator[](const std::string &key)
    {
        if (k_ == kind::null)
            k_ = kind::object;
        if (k_ != kind::object)
            throw std::runtime_error("json: not an object");
        for (auto &m : o_)
            if (m.first == key)
                return m.second;
        o_.emplace_back(key, json());
        return o_.back().second;
    }
    const json &operator[](const std::string &key) const
    {
        if (k_ == kind::object)
            for (auto &m : o_)
                if (m.first == key)
                    return m.second;
        return null_value();
    }
    json &operator[](const char *key) { return (*this)[std::string(key)]; }
    const json &operator[](const char *key) const { return (*this)[std::string(key)]; }
    template <class I, typename std::enable_if<std::is_integral<I>::value, int>::type = 0>
    json &operator[](I idx)
    {
        if (k_ == kind::null)
            k_ = kind::array;
        if (k_ != kind::array)
            throw std::runtime_error("json: not an array");
        const size_t i = (size_t)idx;
        if (i >= a_.size())
            a_.resize(i + 1);
        return a_[i];
    }
    template <class I, typename std::enable_if<std::is_integral<I>::value, int>::type = 0>
    const json &operator[](I idx) const
    {
        const size_t i = (size_t)idx;
        if (k_ != kind::array || i >= a_.size())
            throw std::runtime_error("json: index out of range");
        return a_[i];
    }

    bool contains(const std::string &key) const
    {
        if (k_ != kind::object)
            return false;
        for (auto &m : o_)
            if (m.first == key)
                return true;
        return false;
    }
    size_t size() const
    {
        switch (k_) {
        case kind::null: return 0;
        case kind::array: return a_.size();
        case kind::object: return o_.size();
        default: return 1;
        }
    }

    template <class T> T get() const { return getter<T>::get(*this); }

    template <class T> T value(const std::string &key, const T &def) const
    {
        return contains(key) ? (*this)[key].template get<T>() : def;
    }
    std::string value(const std::string &key, const char *def) const
    {
        return contains(key) ? (*this)[key].template get<std::string>() : std::string(def);
    }

    operator std::string() const { return get<std::string>(); }
    bool operator==(const char *s) const { return k_ == kind::string && s_ == s; }
    bool operator!=(const char *s) const { return !(*this == s); }

    // range-for: an array's elements, an object's values, nothing for null
    class iterator {
    public:
        iterator(const json *arr, size_t i, const std::vector<std::pair<std::string, json>> *obj)
            : arr_(arr), i_(i), obj_(obj)
        {
        }
        const json &operator*() const { return obj_ ? (*obj_)[i_].second : arr_[i_]; }
        iterator &operator++()
        {
            ++i_;
            return *this;
        }
        bool operator!=(const iterator &o) const { return i_ != o.i_; }

    private:
        const json *arr_;
        size_t i_;
        const std::vector<std::pair<std::string, json>> *obj_;
    };
    iterator begin() const
    {
        return iterator(a_.data(), 0, k_ == kind::object ? &o_ : nullptr);
    }
    iterator end() const { return iterator(a_.data(), size_of_range(), k_ == kind::object ? &o_ : nullptr); }

private:
    kind k_ = kind::null;
    bool b_ = false;
    long long i_ = 0;
    unsigned long long u_ = 0;
    double d_ = 0.0;
    std::string s_;
    std::vector<json> a_;
    std::vector<std::pair<std::string, json>> o_;

    size_t size_of_range() const
    {
        return k_ == kind::array ? a_.size() : (k_ == kind::object ? o_.size() : 0);
    }
    static const json &null_value()
    {
        static const json n;
        return n;
    }

    template <class T, class Enable = void> struct getter;

    // ------------------------------------------------------------ parser --
    static void skip_ws(const std::string &t, size_t &at)
    {
        while (at < t.size() && (t[at] == ' ' || t[at] == '\t' || t[at] == '\n' || t[at] == '\r'))
            at++;
    }
    static void expect(const std::string &t, size_t &at, const char *word)
    {
        for (const char *p = word; *p; p++, at++)
            if (at >= t.size() || t[at] != *p)
                throw std::runtime_error("json: bad literal");
    }
    static void put_utf8(std::string &out, unsigned cp)
    {
        if (cp < 0x80) {
            out += (char)cp;
        } else if (cp < 0x800) {
            out += (char)(0xC0 | (cp >> 6));
            out += (char)(0x80 | (cp & 0x3F));
        } else if (cp < 0x10000) {
            out += (char)(0xE0 | (cp >> 12));
            out += (char)(0x80 | ((cp >> 6) & 0x3F));
            out += (char)(0x80 | (cp & 0x3F));
        } else {
            out += (char)(0xF0 | (cp >> 18));
            out += (char)(0x80 | ((cp >> 12) & 0x3F));
            out += (char)(0x80 | ((cp >> 6) & 0x3F));
            out += (char)(0x80 | (cp & 0x3F));
        }
    }
    static unsigned hex4(const std::string &t, size_t &at)
    {
        if (at + 4 > t.size())
            throw std::runtime_error("json: bad escape");
        unsigned v = 0;
        for (int k = 0; k < 4; k++) {
            const char c = t[at++];
            v <<= 4;
            if (c >= '0' && c <= '9')
                v |= (unsigned)(c - '0');
            else if (c >= 'a' && c <= 'f')
                v |= (unsigned)(c - 'a' + 10);
            else if (c >= 'A' && c <= 'F')
                v |= (unsigned)(c - 'A' + 10);
            else
                throw std::runtime_error("json: bad escape");
        }
        return v;
    }
    static std::string parse_string(const std::string &t, size_t &at)
    {
        if (t[at] != '"')
            throw std::runtime_error("json: string expected");
        at++;
        std::string out;
        while (at < t.size() && t[at] != '"') {
            char c = t[at++];
            if (c != '\\') {
                out += c;
                continue;
            }
            if (at >= t.size())
                break;
            c = t[at++];
            switch (c) {
            case '"': out += '"'; break;
            case '\\': out += '\\'; break;
            case '/': out += '/'; break;
            case 'b': out += '\b'; break;
            case 'f': out += '\f'; break;
            case 'n': out += '\n'; break;
            case 'r': out += '\r'; break;
            case 't': out += '\t'; break;
            case 'u': {
                unsigned cp = hex4(t, at);
                if (cp >= 0xD800 && cp < 0xDC00 && at + 6 <= t.size() && t[at] == '\\' && t[at + 1] == 'u') {
                    at += 2;
                    const unsigned lo = hex4(t, at);
                    cp = 0x10000 + ((cp - 0xD800) << 10) + (lo - 0xDC00);
                }
                put_utf8(out, cp);
                break;
            }
            default: throw std::runtime_error("json: bad escape");
            }
        }
        if (at >= t.size())
            throw std::runtime_error("json: unterminated string");
        at++;
        return out;
    }
    static json parse_number(const std::string &t, size_t &at)
    {
        const size_t start = at;
        bool is_float = false;
        if (t[at] == '-')
            at++;
        while (at < t.size()) {
            const char c = t[at];
            if (c >= '0' && c <= '9') {
                at++;
            } else if (c == '.' || c == 'e' || c == 'E' || c == '+' || c == '-') {
                is_float = true;
                at++;
            } else {
                break;
            }
        }
        const std::string num = t.substr(start, at - start);
        json j;
        if (!is_float) {
            errno = 0;
            if (num[0] == '-') {
                const long long v = std::strtoll(num.c_str(), nullptr, 10);
                if (errno == 0) {
                    j.k_ = kind::integer;
                    j.i_ = v;
                    return j;
                }
            } else {
                const unsigned long long v = std::strtoull(num.c_str(), nullptr, 10);
                if (errno == 0) {
                    j.k_ = kind::unsigned_integer;
                    j.u_ = v;
                    return j;
                }
            }
        }
        j.k_ = kind::floating;
        j.d_ = std::strtod(num.c_str(), nullptr);
        return j;
    }
    static json parse_value(const std::string &t, size_t &at)
    {
        skip_ws(t, at);
        if (at >= t.size())
            throw std::runtime_error("json: unexpected end");
        json j;
        const char c = t[at];
        if (c == '{') {
            at++;
            j.k_ = kind::object;
            skip_ws(t, at);
            if (at < t.size() && t[at] == '}') {
                at++;
                return j;
            }
            for (;;) {
                skip_ws(t, at);
                std::string key = parse_string(t, at);
                skip_ws(t, at);
                if (at >= t.size() || t[at] != ':')
                    throw std::runtime_error("json: ':' expected");
                at++;
                json v = parse_value(t, at);
                j.o_.emplace_back(std::move(key), std::move(v));
                skip_ws(t, at);
                if (at < t.size() && t[at] == ',') {
                    at++;
                    continue;
                }
                if (at < t.size() && t[at] == '}') {
                    at++;
                    return j;
                }
                throw std::runtime_error("json: ',' or '}' expected");
            }
        }
        if (c == '[') {
            at++;
            j.k_ = kind::array;
            skip_ws(t, at);
            if (at < t.size() && t[at] == ']') {
                at++;
                return j;
            }
            for (;;) {
                j.a_.push_back(parse_value(t, at));
                skip_ws(t, at);
                if (at < t.size() && t[at] == ',') {
                    at++;
                    continue;
                }
                if (at < t.size() && t[at] == ']') {
                    at++;
                    return j;
                }
                throw std::runtime_error("json: ',' or ']' expected");
            }
        }
        if (c == '"') {
            j.k_ = kind::string;
            j.s_ = parse_string(t, at);
            return j;
        }
        if (c == 't') {
            expect(t, at, "true");
            j.k_ = kind::boolean;
            j.b_ = true;
            return j;
        }
        if (c == 'f') {
            expect(t, at, "false");
            j.k_ = kind::boolean;
            return j;
        }
        if (c == 'n') {
            expect(t, at, "null");
            return j;
        }
        return parse_number(t, at);
    }
};

template <class T> struct json::getter<T, typename std::enable_if<std::is_arithmetic<T>::value>::type> {
    static T get(const json &j)
    {
        switch (j.k_) {
        case kind::integer: return static_cast<T>(j.i_);
        case kind::unsigned_integer: return static_cast<T>(j.u_);
        case kind::floating: return static_cast<T>(j.d_);
        case kind::boolean: return static_cast<T>(j.b_);
        default: throw std::runtime_error("json: number expected");
        }
    }
};
template <> struct json::getter<std::string, void> {
    static std::string get(const json &j)
    {
        if (j.k_ != kind::string)
            throw std::runtime_error("json: string expected");
        return j.s_;
    }
};

} // namespace nlohmann
