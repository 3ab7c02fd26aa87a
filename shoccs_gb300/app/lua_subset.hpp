// lua_subset.hpp -- evaluates the Lua input files of the shoccs command line.
//
// The reference reads its input with a full Lua interpreter (sol2 over Lua, with the base
// and math libraries open: src/app/shoccs.cpp:33-43) and then reads the global table
// `simulation`.  Input files are declarative: nested table constructors, numbers, strings,
// booleans, arithmetic, local and global variables, field assignments and math.* calls.
// This header evaluates exactly that subset:
//
//   statements   [local] name {, name} = exp {, exp};  target.field = exp;  target[exp] = exp;
//                do ... end;  if ... then ... elseif ... else ... end;  numeric for;  while;
//                break;  function calls (print, math.*);  function name(...) ... end
//   expressions  nil true false numbers strings (all quote forms, long brackets) tables
//                or and < > <= >= == ~= .. + - * / // % ^ (right-associative) not # unary -
//                name, .field, [key], calls f(...), f{...}, f"..."
//   functions    function literals and definitions (global, local, a.b.c) with named
//                parameters and return; calls run the body (one result; the enclosing
//                locals are captured by value when the function is defined; 200 levels)
//   math         pi huge maxinteger mininteger abs ceil floor sqrt exp log sin cos tan asin
//                acos atan fmod min max tointeger type modf ult
//   base         print type tostring tonumber string.format
//
// Numbers are doubles (integer-valued ones index array parts and print as integers).  Any
// other construct (generic for, repeat, methods, metatables, goto) is rejected with a
// message naming the line; a loop that runs more than 1e7 iterations is stopped.
#pragma once

#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <functional>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <variant>
#include <vector>

namespace ccs::lua
{
struct error : std::runtime_error {
    using std::runtime_error::runtime_error;
};

struct table;
struct value;
struct fn_body;
// a function defined in the input: where it was defined and its body
struct function_ref {
    std::string where;
    std::shared_ptr<const fn_body> body;
    bool operator==(const function_ref&) const = default;
};
struct builtin {
    std::string name;
    std::function<value(const std::vector<value>&)> fn;
};

struct value {
    std::variant<std::monostate, bool, double, std::string, std::shared_ptr<table>, function_ref,
                 std::shared_ptr<builtin>>
        v;

    value() = default;
    value(bool b) : v{b} {}
    value(double d) : v{d} {}
    value(int i) : v{(double)i} {}
    value(std::string s) : v{std::move(s)} {}
    value(const char* s) : v{std::string{s}} {}
    value(std::shared_ptr<table> t) : v{std::move(t)} {}
    value(function_ref f) : v{std::move(f)} {}
    value(std::shared_ptr<builtin> b) : v{std::move(b)} {}

    bool is_nil() const { return v.index() == 0; }
    bool truthy() const { return !(is_nil() || (v.index() == 1 && !std::get<bool>(v))); }
    const double* number() const { return std::get_if<double>(&v); }
    const std::string* string() const { return std::get_if<std::string>(&v); }
    const bool* boolean() const { return std::get_if<bool>(&v); }
    std::shared_ptr<table> tbl() const
    {
        auto p = std::get_if<std::shared_ptr<table>>(&v);
        return p ? *p : nullptr;
    }
    bool is_function() const { return v.index() == 5 || v.index() == 6; }
    const char* type_name() const
    {
        static const char* names[] = {"nil", "boolean", "number", "string", "table", "function", "function"};
        return names[v.index()];
    }
};

// integer-valued doubles within the exact range are integer keys
inline bool integer_key(double d, long long& k)
{
    if (!(std::fabs(d) < 9.007199254740992e15) || d != std::floor(d)) return false;
    k = (long long)d;
    return true;
}

struct table {
    std::map<long long, value> ints;
    std::map<double, value> reals;
    std::map<std::string, value> strs;
    std::vector<std::pair<value, value>> others; // boolean / table / function keys

    value get(const value& key) const
    {
        if (auto d = key.number()) {
            long long k;
            if (integer_key(*d, k)) {
                auto it = ints.find(k);
                return it == ints.end() ? value{} : it->second;
            }
            auto it = reals.find(*d);
            return it == reals.end() ? value{} : it->second;
        }
        if (auto s = key.string()) {
            auto it = strs.find(*s);
            return it == strs.end() ? value{} : it->second;
        }
        return value{};
    }
    value get(const std::string& key) const { return get(value{key}); }
    value get(const char* key) const { return get(value{std::string{key}}); }
    value get(long long i) const { return get(value{(double)i}); }

    void set(const value& key, value val)
    {
        if (key.is_nil()) throw error("table index is nil");
        if (auto d = key.number()) {
            if (std::isnan(*d)) throw error("table index is NaN");
            long long k;
            if (integer_key(*d, k)) {
                if (val.is_nil()) ints.erase(k);
                else ints[k] = std::move(val);
            } else {
                if (val.is_nil()) reals.erase(*d);
                else reals[*d] = std::move(val);
            }
            return;
        }
        if (auto s = key.string()) {
            if (val.is_nil()) strs.erase(*s);
            else strs[*s] = std::move(val);
            return;
        }
        others.emplace_back(key, std::move(val));
    }
    // the border #t of the array part: n such that t[n] ~= nil and t[n+1] == nil, from 1
    long long length() const
    {
        long long n = 0;
        while (ints.count(n + 1)) ++n;
        return n;
    }
};

inline std::string to_display(const value& v)
{
    if (auto d = v.number()) {
        long long k;
        char buf[64];
        if (integer_key(*d, k)) std::snprintf(buf, sizeof buf, "%lld", k);
        else std::snprintf(buf, sizeof buf, "%.14g", *d);
        return buf;
    }
    if (auto s = v.string()) return *s;
    if (auto b = v.boolean()) return *b ? "true" : "false";
    if (v.is_nil()) return "nil";
    return v.type_name();
}

namespace detail
{
enum class tk { name, number, string, op, eof };
struct token {
    tk kind;
    std::string text; // name, operator, or the string's contents
    double num = 0.0;
    int line = 0;
};

class lexer
{
    const std::string& s_;
    std::string chunk_;
    std::size_t i_ = 0;
    int line_ = 1;

    [[noreturn]] void fail(const std::string& m) const
    {
        throw error(chunk_ + ":" + std::to_string(line_) + ": " + m);
    }
    char peek(std::size_t k = 0) const { return i_ + k < s_.size() ? s_[i_ + k] : '\0'; }

    // "[" "="* "[" ... "]" "="* "]" starting at i_ (on the first '['); -1 when not a long bracket
    int long_level() const
    {
        if (peek() != '[') return -1;
        std::size_t k = 1;
        while (peek(k) == '=') ++k;
        return peek(k) == '[' ? (int)(k - 1) : -1;
    }
    std::string long_string(int level)
    {
        i_ += level + 2;
        if (peek() == '\r' || peek() == '\n') { // a first newline is skipped
            if (peek() == '\n') ++line_;
            ++i_;
        }
        std::string out;
        for (;;) {
            if (i_ >= s_.size()) fail("unfinished long string or comment");
            if (peek() == ']') {
                std::size_t k = 1;
                while (peek(k) == '=') ++k;
                if (peek(k) == ']' && (int)(k - 1) == level) {
                    i_ += k + 1;
                    return out;
                }
            }
            if (peek() == '\n') ++line_;
            out += s_[i_++];
        }
    }
    std::string quoted(char q)
    {
        ++i_;
        std::string out;
        for (;;) {
            const char c = peek();
            if (c == '\0' && i_ >= s_.size()) fail("unfinished string");
            if (c == '\n') fail("unfinished string");
            ++i_;
            if (c == q) return out;
            if (c != '\\') {
                out += c;
                continue;
            }
            const char e = peek();
            ++i_;
            switch (e) {
            case 'n': out += '\n'; break;
            case 't': out += '\t'; break;
            case 'r': out += '\r'; break;
            case 'a': out += '\a'; break;
            case 'b': out += '\b'; break;
            case 'f': out += '\f'; break;
            case 'v': out += '\v'; break;
            case '\\': out += '\\'; break;
            case '"': out += '"'; break;
            case '\'': out += '\''; break;
            case '\n': out += '\n'; ++line_; break;
            default:
                if (e >= '0' && e <= '9') {
                    int v = e - '0';
                    for (int k = 0; k < 2 && peek() >= '0' && peek() <= '9'; k++) v = 10 * v + (s_[i_++] - '0');
                    if (v > 255) fail("decimal escape too large");
                    out += (char)v;
                } else {
                    fail(std::string("invalid escape sequence '\\") + e + "'");
                }
            }
        }
    }

public:
    lexer(const std::string& s, std::string chunk) : s_{s}, chunk_{std::move(chunk)} {}

    std::vector<token> run()
    {
        std::vector<token> out;
        for (;;) {
            // whitespace and comments
            for (;;) {
                const char c = peek();
                if (c == '\n') {
                    ++line_;
                    ++i_;
                } else if (c == ' ' || c == '\t' || c == '\r' || c == '\f' || c == '\v') {
                    ++i_;
                } else if (c == '-' && peek(1) == '-') {
                    i_ += 2;
                    if (const int lv = long_level(); lv >= 0) {
                        long_string(lv);
                    } else {
                        while (i_ < s_.size() && peek() != '\n') ++i_;
                    }
                } else {
                    break;
                }
            }
            if (i_ >= s_.size()) {
                out.push_back({tk::eof, "<eof>", 0.0, line_});
                return out;
            }
            const char c = peek();
            const int line = line_;
            if (std::isalpha((unsigned char)c) || c == '_') {
                std::size_t j = i_;
                while (j < s_.size() && (std::isalnum((unsigned char)s_[j]) || s_[j] == '_')) ++j;
                out.push_back({tk::name, s_.substr(i_, j - i_), 0.0, line});
                i_ = j;
            } else if (std::isdigit((unsigned char)c) || (c == '.' && std::isdigit((unsigned char)peek(1)))) {
                std::size_t j = i_;
                const bool hex = c == '0' && (peek(1) == 'x' || peek(1) == 'X');
                if (hex) j += 2;
                while (j < s_.size()) {
                    const char d = s_[j];
                    const bool expo = hex ? (d == 'p' || d == 'P') : (d == 'e' || d == 'E');
                    if (expo && j + 1 < s_.size() && (s_[j + 1] == '+' || s_[j + 1] == '-')) {
                        j += 2;
                    } else if (std::isxdigit((unsigned char)d) || d == '.' || expo) {
                        if (!hex && std::isalpha((unsigned char)d) && !expo) break;
                        ++j;
                    } else {
                        break;
                    }
                }
                const std::string txt = s_.substr(i_, j - i_);
                char* end = nullptr;
                double v = 0.0;
                if (hex && txt.find_first_of(".pP") == std::string::npos)
                    v = (double)std::strtoull(txt.c_str(), &end, 16);
                else
                    v = std::strtod(txt.c_str(), &end);
                if (!end || *end != '\0') fail("malformed number near '" + txt + "'");
                out.push_back({tk::number, txt, v, line});
                i_ = j;
            } else if (c == '"' || c == '\'') {
                out.push_back({tk::string, quoted(c), 0.0, line});
            } else if (c == '[' && long_level() >= 0) {
                out.push_back({tk::string, long_string(long_level()), 0.0, line});
            } else {
                static const char* ops3[] = {"..."};
                static const char* ops2[] = {"==", "~=", "<=", ">=", "//", "..", "::", "<<", ">>"};
                std::string op;
                for (auto o : ops3)
                    if (s_.compare(i_, 3, o) == 0) op = o;
                if (op.empty())
                    for (auto o : ops2)
                        if (s_.compare(i_, 2, o) == 0) op = o;
                if (op.empty()) {
                    if (std::string("+-*/%^#&~|<>=(){}[];:,.").find(c) == std::string::npos)
                        fail(std::string("unexpected symbol '") + c + "'");
                    op = std::string(1, c);
                }
                out.push_back({tk::op, op, 0.0, line});
                i_ += op.size();
            }
        }
    }
};
} // namespace detail

// a function's parameters, its body (tokens [start, end) of its chunk; t[end] is its `end`)
// and the locals visible where it was defined, captured by value
struct fn_body {
    std::shared_ptr<const std::vector<detail::token>> toks;
    std::vector<std::string> params;
    std::size_t start = 0, end = 0;
    std::string chunk;
    std::vector<std::map<std::string, value>> upvalues;
};

// The interpreter state: the global table (with `math` and `print`) and the chunk's locals.
class state
{
    std::shared_ptr<table> globals_ = std::make_shared<table>();

    struct parser;

public:
    state();
    std::shared_ptr<table> globals() const { return globals_; }
    value get(const std::string& name) const { return globals_->get(name); }

    // run a chunk of source text; `chunk` names it in error messages
    void script(const std::string& source, const std::string& chunk = "script");
    void script_file(const std::string& path)
    {
        std::ifstream f(path, std::ios::binary);
        if (!f) throw error("cannot open " + path);
        std::stringstream ss;
        ss << f.rdbuf();
        script(ss.str(), path);
    }
};

struct state::parser {
    using token = detail::token;
    using tk = detail::tk;

    std::shared_ptr<const std::vector<token>> toks;
    const std::vector<token>& t;
    std::size_t p = 0;
    std::shared_ptr<table> G;
    std::vector<std::map<std::string, value>> scopes{1};
    std::string chunk;
    int depth = 0; // calls of input-defined functions in progress

    parser(std::shared_ptr<const std::vector<token>> tokens, std::shared_ptr<table> g, std::string c)
        : toks{std::move(tokens)}, t{*toks}, G{std::move(g)}, chunk{std::move(c)}
    {
    }
    struct return_signal {
        std::vector<value> values;
    };

    [[noreturn]] void fail(const std::string& m) const
    {
        throw error(chunk + ":" + std::to_string(t[p].line) + ": " + m);
    }
    const token& cur() const { return t[p]; }
    bool is_op(const char* o) const { return cur().kind == tk::op && cur().text == o; }
    bool is_kw(const char* k) const { return cur().kind == tk::name && cur().text == k; }
    void expect_op(const char* o)
    {
        if (!is_op(o)) fail(std::string("'") + o + "' expected near '" + cur().text + "'");
        ++p;
    }
    void expect_kw(const char* k)
    {
        if (!is_kw(k)) fail(std::string("'") + k + "' expected near '" + cur().text + "'");
        ++p;
    }
    static bool keyword(const std::string& s)
    {
        static const char* kws[] = {"and", "break", "do", "else", "elseif", "end", "false", "for",
                                    "function", "goto", "if", "in", "local", "nil", "not", "or",
                                    "repeat", "return", "then", "true", "until", "while"};
        for (auto k : kws)
            if (s == k) return true;
        return false;
    }
    std::string name()
    {
        if (cur().kind != tk::name || keyword(cur().text)) fail("name expected near '" + cur().text + "'");
        return t[p++].text;
    }

    value lookup(const std::string& n) const
    {
        for (auto it = scopes.rbegin(); it != scopes.rend(); ++it)
            if (auto f = it->find(n); f != it->end()) return f->second;
        return G->get(n);
    }
    void assign_name(const std::string& n, value v)
    {
        for (auto it = scopes.rbegin(); it != scopes.rend(); ++it)
            if (auto f = it->find(n); f != it->end()) {
                f->second = std::move(v);
                return;
            }
        G->set(value{n}, std::move(v));
    }

    // ---- statements ----
    void block_until(const char* end_kw)
    {
        while (!(cur().kind == tk::eof || (end_kw && is_kw(end_kw)))) statement();
    }

    // ---- control flow ----
    struct break_signal {
    };
    bool at_kw(std::size_t q, const char* k) const { return t[q].kind == tk::name && t[q].text == k; }
    // from q (just inside a block), the index of the first of `stops` (end, else, elseif)
    // at nesting depth 0
    std::size_t scan_block(std::size_t q, bool if_branch) const
    {
        int depth = 0;
        for (; t[q].kind != tk::eof; ++q) {
            if (t[q].kind != tk::name) continue;
            const std::string& w = t[q].text;
            if (depth == 0 && (w == "end" || (if_branch && (w == "else" || w == "elseif")))) return q;
            if (w == "function" || w == "if" || w == "do" || w == "repeat") ++depth;
            else if (w == "end" || w == "until") --depth;
        }
        throw error(chunk + ":" + std::to_string(t[q].line) + ": 'end' expected");
    }
    // run the statements of [p, stop) in a new scope
    void run_block(std::size_t stop)
    {
        scopes.emplace_back();
        try {
            while (p < stop) statement();
        } catch (...) {
            scopes.pop_back();
            throw;
        }
        scopes.pop_back();
        if (p != stop) fail("unexpected '" + cur().text + "'");
    }
    static constexpr long long max_iterations = 10000000;

    void if_statement()
    {
        // if cond then block {elseif cond then block} [else block] end
        bool done = false;
        for (;;) {
            const bool is_else = is_kw("else");
            ++p; // if / elseif / else
            bool take = false;
            if (!is_else) {
                // after a taken branch the remaining conditions are not evaluated (Lua runs
                // none of their calls or indexing)
                if (done) {
                    skip_expr();
                    expect_kw("then");
                } else {
                    const value c = expr();
                    expect_kw("then");
                    take = c.truthy();
                }
            } else {
                take = !done;
            }
            const std::size_t stop = scan_block(p, true);
            if (take) {
                run_block(stop);
                done = true;
            }
            p = stop;
            if (is_kw("end")) {
                ++p;
                return;
            }
            if (is_else) fail("'end' expected near '" + cur().text + "'");
        }
    }

    void for_statement()
    {
        ++p; // for
        const std::string var = name();
        if (!is_op("=")) fail("only numeric for loops are supported");
        ++p;
        const double a = num(expr(), "for initial value");
        expect_op(",");
        const double b = num(expr(), "for limit");
        double step = 1.0;
        if (is_op(",")) {
            ++p;
            step = num(expr(), "for step");
        }
        if (step == 0) fail("'for' step is zero");
        expect_kw("do");
        const std::size_t body = p, stop = scan_block(p, false);
        long long n = 0;
        try {
            for (double v = a; step > 0 ? v <= b : v >= b; v += step) {
                if (++n > max_iterations) fail("loop runs too long");
                p = body;
                scopes.push_back({{var, value{v}}});
                try {
                    run_block(stop);
                } catch (...) {
                    scopes.pop_back();
                    throw;
                }
                scopes.pop_back();
            }
        } catch (const break_signal&) {
        }
        p = stop + 1;
    }

    void while_statement()
    {
        ++p; // while
        const std::size_t cond = p;
        bool go = expr().truthy();
        expect_kw("do");
        const std::size_t body = p, stop = scan_block(p, false);
        long long n = 0;
        try {
            while (go) {
                if (++n > max_iterations) fail("loop runs too long");
                p = body;
                run_block(stop);
                p = cond;
                go = expr().truthy();
                expect_kw("do");
            }
        } catch (const break_signal&) {
        }
        p = stop + 1;
    }

    void statement()
    {
        if (is_op(";")) {
            ++p;
            return;
        }
        if (is_kw("if")) {
            if_statement();
            return;
        }
        if (is_kw("for")) {
            for_statement();
            return;
        }
        if (is_kw("while")) {
            while_statement();
            return;
        }
        if (is_kw("break")) {
            ++p;
            throw break_signal{};
        }
        if (is_kw("return")) {
            ++p;
            std::vector<value> v;
            if (!(cur().kind == tk::eof || is_op(";") || is_kw("end") || is_kw("else") || is_kw("elseif") ||
                  is_kw("until")))
                v = exprlist();
            if (is_op(";")) ++p;
            throw return_signal{std::move(v)};
        }
        if (is_kw("local")) {
            ++p;
            if (is_kw("function")) {
                ++p;
                const std::string n = name();
                scopes.back()[n] = skip_function_body(n, true);
                return;
            }
            std::vector<std::string> names{name()};
            while (is_op(",")) {
                ++p;
                names.push_back(name());
            }
            if (is_op("<")) fail("local attributes are not supported");
            std::vector<value> vals;
            if (is_op("=")) {
                ++p;
                vals = exprlist();
            }
            for (std::size_t k = 0; k < names.size(); k++)
                scopes.back()[names[k]] = k < vals.size() ? vals[k] : value{};
            return;
        }
        if (is_kw("do")) {
            ++p;
            scopes.emplace_back();
            block_until("end");
            expect_kw("end");
            scopes.pop_back();
            return;
        }
        if (is_kw("function")) {
            ++p;
            // function a.b.c(...) ... end: assign an opaque function to the field
            std::string n = name();
            std::shared_ptr<table> holder;
            std::string field;
            while (is_op(".")) {
                ++p;
                value base = holder ? holder->get(field) : lookup(n);
                auto tb = base.tbl();
                if (!tb) fail("attempt to index a " + std::string(base.type_name()) + " value");
                holder = tb;
                field = name();
            }
            if (is_op(":")) fail("method definitions are not supported");
            value f = skip_function_body(n);
            if (holder) holder->set(value{field}, f);
            else assign_name(n, f);
            return;
        }
        if (cur().kind == tk::name && !keyword(cur().text)) {
            // assignment or call statement
            struct target {
                std::string name;
                std::shared_ptr<table> tbl;
                value key;
            };
            std::vector<target> targets;
            auto parse_target = [&](bool& was_call) {
                std::string n = name();
                value v = lookup(n);
                target tg{n, nullptr, {}};
                was_call = false;
                for (;;) {
                    if (is_op(".") || is_op("[")) {
                        value key;
                        if (is_op(".")) {
                            ++p;
                            key = value{name()};
                        } else {
                            ++p;
                            key = expr();
                            expect_op("]");
                        }
                        value base = tg.tbl ? tg.tbl->get(tg.key) : lookup(tg.name);
                        auto tb = base.tbl();
                        if (!tb) fail("attempt to index a " + std::string(base.type_name()) + " value");
                        tg.tbl = tb;
                        tg.key = key;
                    } else if (is_op("(") || is_op("{") || cur().kind == tk::string) {
                        value fn = tg.tbl ? tg.tbl->get(tg.key) : lookup(tg.name);
                        call(fn, args());
                        was_call = true;
                        tg = target{"", nullptr, {}};
                        // a call result can be indexed further only in an expression
                        if (is_op(".") || is_op("[") || is_op("(")) fail("complex call statements are not supported");
                        return tg;
                    } else if (is_op(":")) {
                        fail("method calls are not supported");
                    } else {
                        return tg;
                    }
                }
            };
            bool was_call = false;
            targets.push_back(parse_target(was_call));
            if (was_call) return;
            while (is_op(",")) {
                ++p;
                targets.push_back(parse_target(was_call));
                if (was_call) fail("syntax error near '" + cur().text + "'");
            }
            expect_op("=");
            std::vector<value> vals = exprlist();
            for (std::size_t k = 0; k < targets.size(); k++) {
                value v = k < vals.size() ? vals[k] : value{};
                if (targets[k].tbl) targets[k].tbl->set(targets[k].key, std::move(v));
                else assign_name(targets[k].name, std::move(v));
            }
            return;
        }
        fail("unsupported statement near '" + cur().text + "'");
    }

    // function literal / definition: skip the parameter list and the body up to its `end`
    // function body: parameters, then the statements up to the matching `end`; `self_name`
    // (a `local function`) is visible inside its own body
    value skip_function_body(const std::string& n, bool self_visible = false)
    {
        const int line = cur().line;
        auto body = std::make_shared<fn_body>();
        expect_op("(");
        while (!is_op(")")) {
            if (is_op("...")) fail("varargs are not supported");
            body->params.push_back(name());
            if (is_op(",")) ++p;
            else if (!is_op(")")) fail("')' expected near '" + cur().text + "'");
        }
        ++p;
        body->start = p;
        int nest = 1;
        while (nest > 0) {
            if (cur().kind == tk::eof) fail("'end' expected (to close function at line " + std::to_string(line) + ")");
            if (cur().kind == tk::name) {
                const std::string& w = cur().text;
                if (w == "function" || w == "if" || w == "do" || w == "repeat") ++nest;
                else if (w == "end" || w == "until") --nest;
            }
            ++p;
        }
        body->end = p - 1;
        body->toks = toks;
        body->chunk = chunk;
        body->upvalues = scopes;
        const value f{function_ref{chunk + ":" + std::to_string(line) + (n.empty() ? "" : " " + n), body}};
        if (self_visible) body->upvalues.back()[n] = f; // recursion (a reference cycle, kept)
        return f;
    }

    // ---- expressions ----
    std::vector<value> exprlist()
    {
        std::vector<value> v{expr()};
        while (is_op(",")) {
            ++p;
            v.push_back(expr());
        }
        return v;
    }

    double num(const value& v, const char* what) const
    {
        if (auto d = v.number()) return *d;
        if (auto s = v.string()) { // string arithmetic coercion
            char* end = nullptr;
            const double d = std::strtod(s->c_str(), &end);
            if (end && *end == '\0' && !s->empty()) return d;
        }
        fail(std::string("attempt to perform arithmetic (") + what + ") on a " + v.type_name() + " value");
    }

    static int prec_left(const std::string& op)
    {
        if (op == "or") return 1;
        if (op == "and") return 2;
        if (op == "<" || op == ">" || op == "<=" || op == ">=" || op == "~=" || op == "==") return 3;
        if (op == "..") return 9; // right associative
        if (op == "+" || op == "-") return 10;
        if (op == "*" || op == "/" || op == "//" || op == "%") return 11;
        if (op == "^") return 14; // right associative
        return -1;
    }
    static int prec_right(const std::string& op)
    {
        if (op == "..") return 8;
        if (op == "^") return 13;
        return prec_left(op);
    }
    std::string binop() const
    {
        if (cur().kind == tk::op && prec_left(cur().text) > 0) return cur().text;
        if (cur().kind == tk::name && (cur().text == "and" || cur().text == "or")) return cur().text;
        return {};
    }

    value expr(int limit = 0)
    {
        value lhs;
        if (is_kw("not") || is_op("-") || is_op("#")) {
            const std::string op = t[p++].text;
            value v = expr(12); // unary priority
            if (op == "not") lhs = value{!v.truthy()};
            else if (op == "-") lhs = value{-num(v, "unm")};
            else {
                if (auto s = v.string()) lhs = value{(double)s->size()};
                else if (auto tb = v.tbl()) lhs = value{(double)tb->length()};
                else fail(std::string("attempt to get length of a ") + v.type_name() + " value");
            }
        } else if (is_op("~")) {
            fail("bitwise operators are not supported");
        } else {
            lhs = simple();
        }
        for (;;) {
            const std::string op = binop();
            if (op.empty() || prec_left(op) <= limit) return lhs;
            ++p;
            if (op == "and" || op == "or") {
                // short circuit: when the left operand decides the result (false or nil for
                // `and`, anything else for `or`) the right one is parsed but not evaluated
                if (op == "and" ? !lhs.truthy() : lhs.truthy()) skip_expr(prec_right(op));
                else lhs = expr(prec_right(op));
                continue;
            }
            value rhs = expr(prec_right(op));
            lhs = arith(op, lhs, rhs);
        }
    }

    // ---- skipping an expression without evaluating it (short-circuit operands, the
    // conditions after a taken branch): the same grammar as expr(), tokens only ----
    void skip_balanced(const char* open, const char* close)
    {
        int nest = 0;
        do {
            if (cur().kind == tk::eof) fail(std::string("'") + close + "' expected");
            if (is_op(open)) ++nest;
            else if (is_op(close)) --nest;
            ++p;
        } while (nest > 0);
    }
    void skip_function_literal()
    {
        const int line = cur().line;
        ++p; // function
        skip_balanced("(", ")");
        int nest = 1;
        while (nest > 0) {
            if (cur().kind == tk::eof) fail("'end' expected (to close function at line " + std::to_string(line) + ")");
            if (cur().kind == tk::name) {
                const std::string& w = cur().text;
                if (w == "function" || w == "if" || w == "do" || w == "repeat") ++nest;
                else if (w == "end" || w == "until") --nest;
            }
            ++p;
        }
    }
    void skip_simple()
    {
        if (cur().kind == tk::number || cur().kind == tk::string || is_kw("nil") || is_kw("true") ||
            is_kw("false") || is_op("...")) {
            ++p;
            return;
        }
        if (is_kw("function")) {
            skip_function_literal();
            return;
        }
        if (is_op("{")) {
            skip_balanced("{", "}");
            return;
        }
        if (is_op("(")) {
            skip_balanced("(", ")");
        } else {
            name();
        }
        for (;;) { // suffixes: fields, indexing, calls
            if (is_op(".") || is_op(":")) {
                ++p;
                name();
            } else if (is_op("[")) {
                skip_balanced("[", "]");
            } else if (is_op("(")) {
                skip_balanced("(", ")");
            } else if (is_op("{")) {
                skip_balanced("{", "}");
            } else if (cur().kind == tk::string) {
                ++p;
            } else {
                return;
            }
        }
    }
    void skip_expr(int limit = 0)
    {
        if (is_kw("not") || is_op("-") || is_op("#")) {
            ++p;
            skip_expr(12);
        } else {
            skip_simple();
        }
        for (;;) {
            const std::string op = binop();
            if (op.empty() || prec_left(op) <= limit) return;
            ++p;
            skip_expr(prec_right(op));
        }
    }

    value arith(const std::string& op, const value& a, const value& b) const
    {
        if (op == "==" || op == "~=") {
            bool eq = false;
            if (a.v.index() == b.v.index()) {
                if (auto x = a.number()) eq = *x == *b.number();
                else if (auto s = a.string()) eq = *s == *b.string();
                else if (auto bo = a.boolean()) eq = *bo == *b.boolean();
                else if (a.is_nil()) eq = true;
                else if (auto tb = a.tbl()) eq = tb == b.tbl();
                else eq = false;
            }
            return value{op == "==" ? eq : !eq};
        }
        if (op == "<" || op == ">" || op == "<=" || op == ">=") {
            if (a.string() && b.string()) {
                const int c = a.string()->compare(*b.string());
                return value{op == "<" ? c < 0 : op == ">" ? c > 0 : op == "<=" ? c <= 0 : c >= 0};
            }
            if (!a.number() || !b.number())
                fail(std::string("attempt to compare ") + a.type_name() + " with " + b.type_name());
            const double x = *a.number(), y = *b.number();
            return value{op == "<" ? x < y : op == ">" ? x > y : op == "<=" ? x <= y : x >= y};
        }
        if (op == "..") {
            auto piece = [&](const value& v) {
                if (!v.number() && !v.string())
                    fail(std::string("attempt to concatenate a ") + v.type_name() + " value");
                return to_display(v);
            };
            return value{piece(a) + piece(b)};
        }
        const double x = num(a, op.c_str()), y = num(b, op.c_str());
        if (op == "+") return value{x + y};
        if (op == "-") return value{x - y};
        if (op == "*") return value{x * y};
        if (op == "/") return value{x / y};
        if (op == "^") return value{std::pow(x, y)};
        if (op == "//") return value{std::floor(x / y)};
        // %: a - floor(a/b)*b, with the result taking the sign of b
        double m = std::fmod(x, y);
        if (m != 0 && ((m < 0) != (y < 0))) m += y;
        return value{m};
    }

    std::vector<value> args()
    {
        if (cur().kind == tk::string) return {value{t[p++].text}};
        if (is_op("{")) return {table_ctor()};
        expect_op("(");
        std::vector<value> a;
        if (!is_op(")")) a = exprlist();
        expect_op(")");
        return a;
    }

    value call(const value& fn, const std::vector<value>& a) const
    {
        if (auto b = std::get_if<std::shared_ptr<builtin>>(&fn.v)) {
            try {
                return (*b)->fn(a);
            } catch (const error& e) {
                fail("bad argument to '" + (*b)->name + "': " + e.what());
            }
        }
        if (auto f = std::get_if<function_ref>(&fn.v); f && f->body) {
            if (depth >= 200) fail("stack overflow (calls nested more than 200 deep)");
            const fn_body& b = *f->body;
            parser sub(b.toks, G, b.chunk);
            sub.depth = depth + 1;
            sub.scopes = b.upvalues;
            std::map<std::string, value> args;
            for (std::size_t i = 0; i < b.params.size(); i++) args[b.params[i]] = i < a.size() ? a[i] : value{};
            sub.scopes.push_back(std::move(args));
            sub.p = b.start;
            try {
                while (sub.p < b.end) sub.statement();
            } catch (const return_signal& r) {
                return r.values.empty() ? value{} : r.values[0];
            } catch (const break_signal&) {
                throw error(b.chunk + ": break outside a loop");
            }
            return value{};
        }
        fail(std::string("attempt to call a ") + fn.type_name() + " value");
    }

    value simple()
    {
        const token& c = cur();
        if (c.kind == tk::number) {
            ++p;
            return value{c.num};
        }
        if (c.kind == tk::string) {
            ++p;
            return value{c.text};
        }
        if (is_kw("nil")) {
            ++p;
            return value{};
        }
        if (is_kw("true") || is_kw("false")) {
            ++p;
            return value{c.text == "true"};
        }
        if (is_op("...")) fail("varargs are not supported");
        if (is_kw("function")) {
            ++p;
            return skip_function_body("");
        }
        if (is_op("{")) return table_ctor();
        return suffixed();
    }

    value suffixed()
    {
        value v;
        if (is_op("(")) {
            ++p;
            v = expr();
            expect_op(")");
        } else {
            v = lookup(name());
        }
        for (;;) {
            if (is_op(".")) {
                ++p;
                const std::string k = name();
                auto tb = v.tbl();
                if (!tb) fail("attempt to index a " + std::string(v.type_name()) + " value (field '" + k + "')");
                v = tb->get(k);
            } else if (is_op("[")) {
                ++p;
                value k = expr();
                expect_op("]");
                auto tb = v.tbl();
                if (!tb) fail("attempt to index a " + std::string(v.type_name()) + " value");
                v = tb->get(k);
            } else if (is_op("(") || is_op("{") || cur().kind == tk::string) {
                v = call(v, args());
            } else if (is_op(":")) {
                fail("method calls are not supported");
            } else {
                return v;
            }
        }
    }

    value table_ctor()
    {
        expect_op("{");
        auto tb = std::make_shared<table>();
        long long next = 1;
        while (!is_op("}")) {
            if (is_op("[")) {
                ++p;
                value k = expr();
                expect_op("]");
                expect_op("=");
                tb->set(k, expr());
            } else if (cur().kind == tk::name && !keyword(cur().text) && t[p + 1].kind == tk::op &&
                       t[p + 1].text == "=") {
                const std::string k = name();
                ++p; // '='
                tb->set(value{k}, expr());
            } else {
                tb->set(value{(double)next++}, expr());
            }
            if (is_op(",") || is_op(";")) ++p;
            else if (!is_op("}")) fail("'}' expected near '" + cur().text + "'");
        }
        ++p;
        return value{tb};
    }
};

inline state::state()
{
    auto math = std::make_shared<table>();
    auto fn1 = [&](const char* n, double (*f)(double)) {
        math->set(value{n}, value{std::make_shared<builtin>(builtin{std::string("math.") + n, [f](const std::vector<value>& a) {
                                     if (a.empty() || !a[0].number()) throw error("number expected");
                                     return value{f(*a[0].number())};
                                 }})});
    };
    fn1("abs", [](double x) { return std::fabs(x); });
    fn1("ceil", [](double x) { return std::ceil(x); });
    fn1("floor", [](double x) { return std::floor(x); });
    fn1("sqrt", [](double x) { return std::sqrt(x); });
    fn1("exp", [](double x) { return std::exp(x); });
    fn1("sin", [](double x) { return std::sin(x); });
    fn1("cos", [](double x) { return std::cos(x); });
    fn1("tan", [](double x) { return std::tan(x); });
    fn1("asin", [](double x) { return std::asin(x); });
    fn1("acos", [](double x) { return std::acos(x); });
    auto put = [&](const char* n, std::function<value(const std::vector<value>&)> f) {
        math->set(value{n}, value{std::make_shared<builtin>(builtin{std::string("math.") + n, std::move(f)})});
    };
    auto nums = [](const std::vector<value>& a, std::size_t n) {
        if (a.size() < n) throw error("number expected");
        for (std::size_t k = 0; k < n; k++)
            if (!a[k].number()) throw error("number expected");
    };
    put("log", [nums](const std::vector<value>& a) {
        nums(a, 1);
        const double x = *a[0].number();
        if (a.size() > 1 && a[1].number()) {
            const double b = *a[1].number();
            return value{b == 2.0 ? std::log2(x) : b == 10.0 ? std::log10(x) : std::log(x) / std::log(b)};
        }
        return value{std::log(x)};
    });
    put("atan", [nums](const std::vector<value>& a) {
        nums(a, 1);
        const double x = a.size() > 1 && a[1].number() ? *a[1].number() : 1.0;
        return value{std::atan2(*a[0].number(), x)};
    });
    put("fmod", [nums](const std::vector<value>& a) {
        nums(a, 2);
        return value{std::fmod(*a[0].number(), *a[1].number())};
    });
    put("modf", [nums](const std::vector<value>& a) {
        nums(a, 1);
        double ip = 0.0;
        return value{std::modf(*a[0].number(), &ip)};
    });
    put("min", [nums](const std::vector<value>& a) {
        nums(a, 1);
        double m = *a[0].number();
        for (std::size_t k = 1; k < a.size(); k++) {
            if (!a[k].number()) throw error("number expected");
            m = std::fmin(m, *a[k].number());
        }
        return value{m};
    });
    put("max", [nums](const std::vector<value>& a) {
        nums(a, 1);
        double m = *a[0].number();
        for (std::size_t k = 1; k < a.size(); k++) {
            if (!a[k].number()) throw error("number expected");
            m = std::fmax(m, *a[k].number());
        }
        return value{m};
    });
    put("tointeger", [](const std::vector<value>& a) {
        long long k;
        if (!a.empty() && a[0].number() && integer_key(*a[0].number(), k)) return a[0];
        return value{};
    });
    put("type", [](const std::vector<value>& a) {
        if (a.empty() || !a[0].number()) return value{};
        long long k;
        return value{integer_key(*a[0].number(), k) ? "integer" : "float"};
    });
    put("ult", [nums](const std::vector<value>& a) {
        nums(a, 2);
        return value{(unsigned long long)(long long)*a[0].number() < (unsigned long long)(long long)*a[1].number()};
    });
    math->set(value{"pi"}, value{3.141592653589793});
    math->set(value{"huge"}, value{HUGE_VAL});
    math->set(value{"maxinteger"}, value{9.223372036854775807e18});
    math->set(value{"mininteger"}, value{-9.223372036854775808e18});
    globals_->set(value{"math"}, value{math});
    // base and string functions: type, tostring, tonumber, string.format (%d %i %u %c %x %X %o
    // %e %E %f %g %G %q-less subset, %s, %%)
    auto gput = [&](std::shared_ptr<table> tb, const char* n, std::function<value(const std::vector<value>&)> f) {
        tb->set(value{n}, value{std::make_shared<builtin>(builtin{n, std::move(f)})});
    };
    gput(globals_, "type", [](const std::vector<value>& a) {
        return value{a.empty() ? "nil" : a[0].type_name()};
    });
    gput(globals_, "tostring", [](const std::vector<value>& a) { return value{a.empty() ? "nil" : to_display(a[0])}; });
    gput(globals_, "tonumber", [](const std::vector<value>& a) {
        if (a.empty()) throw error("value expected");
        if (a[0].number()) return a[0];
        if (auto str = a[0].string()) {
            // a decimal or hexadecimal numeral with optional surrounding white space; Lua's
            // tonumber has no inf or nan numerals
            const char* b = str->c_str();
            while (std::isspace((unsigned char)*b)) ++b;
            const char* q = (*b == '+' || *b == '-') ? b + 1 : b;
            if (std::isdigit((unsigned char)*q) || (*q == '.' && std::isdigit((unsigned char)q[1]))) {
                char* end = nullptr;
                const double d = std::strtod(b, &end);
                if (end && end != b) {
                    while (std::isspace((unsigned char)*end)) ++end;
                    if (*end == '\0') return value{d};
                }
            }
        }
        return value{};
    });
    auto strlib = std::make_shared<table>();
    gput(strlib, "format", [](const std::vector<value>& a) {
        if (a.empty() || !a[0].string()) throw error("format string expected");
        const std::string& f = *a[0].string();
        std::string out;
        std::size_t arg = 1;
        for (std::size_t i = 0; i < f.size(); i++) {
            if (f[i] != '%') {
                out += f[i];
                continue;
            }
            if (++i >= f.size()) throw error("invalid conversion '%' to 'format'");
            if (f[i] == '%') {
                out += '%';
                continue;
            }
            std::string spec = "%";
            while (i < f.size() && std::strchr("-+ #0123456789.", f[i])) spec += f[i++];
            if (i >= f.size()) throw error("invalid conversion to 'format'");
            const char c = f[i];
            if (arg >= a.size()) throw error("bad argument #" + std::to_string(arg + 1) + " to 'format' (no value)");
            const value& v = a[arg++];
            const std::string bad = "bad argument #" + std::to_string(arg) + " to 'format' ";
            std::string buf;
            auto put = [&](const std::string& fmt, auto x) {
                const int n = std::snprintf(nullptr, 0, fmt.c_str(), x);
                if (n < 0) throw error(bad + "(invalid conversion)");
                buf.assign((std::size_t)n + 1, '\0');
                std::snprintf(buf.data(), buf.size(), fmt.c_str(), x);
                buf.resize((std::size_t)n);
            };
            if (c == 's') {
                const std::string str = to_display(v);
                put(spec + "s", str.c_str());
            } else if (std::strchr("dicxXou", c)) {
                if (!v.number()) throw error(bad + "(number expected, got " + v.type_name() + ")");
                const double x = *v.number();
                // the integer conversions take numbers with an exact integer value in range
                if (!(x == std::floor(x)) || !(x >= -9.223372036854775808e18 && x < 9.223372036854775808e18))
                    throw error(bad + "(number has no integer representation)");
                if (c == 'c') put(spec + "c", (int)(long long)x);
                else put(spec + "ll" + (c == 'i' ? 'd' : c), (long long)x);
            } else if (std::strchr("eEfgGaA", c)) {
                if (!v.number()) throw error(bad + "(number expected, got " + v.type_name() + ")");
                put(spec + c, *v.number());
            } else {
                throw error(std::string("invalid conversion '%") + c + "' to 'format'");
            }
            out += buf;
        }
        return value{out};
    });
    globals_->set(value{"string"}, value{strlib});
    globals_->set(value{"print"}, value{std::make_shared<builtin>(builtin{"print", [](const std::vector<value>& a) {
                                           std::string line;
                                           for (std::size_t k = 0; k < a.size(); k++)
                                               line += (k ? "\t" : "") + to_display(a[k]);
                                           std::printf("%s\n", line.c_str());
                                           return value{};
                                       }})});
}

inline void state::script(const std::string& source, const std::string& chunk)
{
    std::string text = source;
    if (text.rfind("#", 0) == 0) { // a first line starting with '#' is skipped
        const std::size_t nl = text.find('\n');
        text = nl == std::string::npos ? "" : text.substr(nl);
    }
    parser ps(std::make_shared<const std::vector<detail::token>>(detail::lexer(text, chunk).run()), globals_,
              chunk);
    try {
        ps.block_until(nullptr);
    } catch (const parser::break_signal&) {
        throw error(chunk + ": break outside a loop");
    } catch (const parser::return_signal&) {
        // a chunk may end with return
    }
}
} // namespace ccs::lua
