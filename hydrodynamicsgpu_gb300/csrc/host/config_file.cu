// config_file.cu -- hgpu_config from a config.lua-style file (host code only).
//
// The reference reads its run configuration from a Lua script through LuaCxx
// (src/HydroGPUApp.cpp:157-208, :330; src/Solver/Solver.cpp:196-197, 285-307;
// res/config.lua:26-94).  No Lua interpreter exists on this path, so this file
// evaluates the part of Lua such a script's settings are written in:
//
//   statement  := target '=' expr [';']
//   target     := Name { '.' Name | '[' expr ']' }
//   expr       := arithmetic over numbers (+ - * / % ^, unary -, parentheses),
//                 'string' / "string", true, false, nil, table constructors
//                 { expr, Name = expr, [expr] = expr } and reads of names already
//                 assigned (including math.pi and math.huge)
//   comments   := -- to the end of the line, --[[ ... ]] and --[==[ ... ]==]
//
// Anything else (function calls such as require, if/for/function blocks, local,
// string concatenation, comparisons) cannot be evaluated without running Lua and
// is rejected with HGPU_ERR_CONFIG and the line it is on.  Every assignment is
// evaluated, whatever its key, so a malformed value anywhere is an error.
//
// Keys that set the configuration, with the reference's readers:
//   solverName      EulerRoe | EulerHLLC | EulerHLL        (HydroGPUApp.cpp:330-348)
//   integratorName  ForwardEuler, RungeKutta2, ...         (Solver.cpp:178-204)
//   slopeLimiter    DonorCell ... BarthJespersen           (Solver.cpp:285-287)
//   size, xmin, xmax            {x, y, z}                  (HydroGPUApp.cpp:166-170)
//   boundaryMethods {{min=, max=}, ...}                    (HydroGPUApp.cpp:172-181, 495-511)
//   cfl (a C float), useFixedDT, fixedDT                   (HydroGPUApp.cpp:204-206)
//   useGravity, gaussSeidelMaxIter                         (HydroGPUApp.cpp:207-208)
//   defs.idealGas_heatCapacityRatio, defs.selfGrav_gravitationalConstant
//                                                          (Solver.cpp:289-299)
// The reference reads the limiter from `slopeLimiter` while its shipped config.lua
// assigns `slopeLimiterName` (config.lua:26), so that assignment never reaches the
// solver and Superbee stays in force; the same holds here: `slopeLimiterName` is
// evaluated and ignored.  Keys absent from the file keep hgpu_config_default's
// values, except solverName, whose reference default ("EulerBurgers",
// HydroGPUApp.cpp:67) is not a solver of this path: a file without it is refused
// with HGPU_ERR_UNSUPPORTED, as an unknown solver name is refused by the reference
// (HydroGPUApp.cpp:346-348).
#include <cctype>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../../../include/hgpu/hgpu.h"

namespace hgpu {
void setLastError(const std::string& msg);
}

namespace {

struct Table;

struct Value {
    enum Kind { NIL, BOOL, NUMBER, STRING, TABLE } kind = NIL;
    bool b = false;
    double n = 0;
    std::string s;
    std::shared_ptr<Table> t;
};

// Lua table: integer-valued number keys and string keys (the only kinds a settings
// script uses); a number key that is an integer is stored as such
struct Table {
    std::map<long long, Value> arr;
    std::map<std::string, Value> hash;
};

struct ParseError {
    int status;
    std::string msg;
};

class Reader {
public:
    explicit Reader(const std::string& text) : src_(text) {}

    std::map<std::string, Value> globals;

    void run() {
        auto math = std::make_shared<Table>();
        Value pi, huge;
        pi.kind = huge.kind = Value::NUMBER;
        pi.n = 3.14159265358979323846;
        huge.n = HUGE_VAL;
        math->hash["pi"] = pi;
        math->hash["huge"] = huge;
        Value m;
        m.kind = Value::TABLE;
        m.t = math;
        globals["math"] = m;
        next();
        while (tok_.kind != T_EOF) statement();
    }

private:
    enum TokKind { T_EOF, T_NAME, T_NUMBER, T_STRING, T_OP };
    struct Tok {
        TokKind kind = T_EOF;
        std::string text;
        double num = 0;
        int line = 1;
    };

    const std::string& src_;
    size_t pos_ = 0;
    int line_ = 1;
    Tok tok_;

    [[noreturn]] void error(const std::string& what, int line = -1) const {
        throw ParseError{HGPU_ERR_CONFIG, "config line " + std::to_string(line < 0 ? tok_.line : line) + ": " + what};
    }

    // --[[ ... ]] / --[==[ ... ]==]: level = number of '=' between the brackets
    bool longBracket(size_t at, int& level) const {
        if (at >= src_.size() || src_[at] != '[') return false;
        size_t k = at + 1;
        level = 0;
        while (k < src_.size() && src_[k] == '=') ++level, ++k;
        return k < src_.size() && src_[k] == '[';
    }

    void skipSpaceAndComments() {
        for (;;) {
            while (pos_ < src_.size() && (src_[pos_] == ' ' || src_[pos_] == '\t' || src_[pos_] == '\r' ||
                                          src_[pos_] == '\n' || src_[pos_] == '\f' || src_[pos_] == '\v')) {
                if (src_[pos_] == '\n') ++line_;
                ++pos_;
            }
            if (pos_ + 1 < src_.size() && src_[pos_] == '-' && src_[pos_ + 1] == '-') {
                int level;
                if (longBracket(pos_ + 2, level)) {
                    std::string close = "]" + std::string(level, '=') + "]";
                    size_t end = src_.find(close, pos_ + 2);
                    if (end == std::string::npos) error("unfinished long comment", line_);
                    for (size_t k = pos_; k < end; ++k)
                        if (src_[k] == '\n') ++line_;
                    pos_ = end + close.size();
                } else {
                    while (pos_ < src_.size() && src_[pos_] != '\n') ++pos_;
                }
                continue;
            }
            return;
        }
    }

    void next() {
        skipSpaceAndComments();
        tok_ = Tok();
        tok_.line = line_;
        if (pos_ >= src_.size()) return;
        const char c = src_[pos_];
        if (std::isalpha((unsigned char)c) || c == '_') {
            size_t b = pos_;
            while (pos_ < src_.size() && (std::isalnum((unsigned char)src_[pos_]) || src_[pos_] == '_')) ++pos_;
            tok_.kind = T_NAME;
            tok_.text = src_.substr(b, pos_ - b);
            return;
        }
        if (std::isdigit((unsigned char)c) || (c == '.' && pos_ + 1 < src_.size() &&
                                               std::isdigit((unsigned char)src_[pos_ + 1]))) {
            // Lua numerals: decimal with optional fraction and exponent, or 0x hexadecimal;
            // converted as Lua does (strtod in the C locale)
            size_t b = pos_;
            if (c == '0' && pos_ + 1 < src_.size() && (src_[pos_ + 1] == 'x' || src_[pos_ + 1] == 'X')) {
                pos_ += 2;
                while (pos_ < src_.size() && (std::isxdigit((unsigned char)src_[pos_]) || src_[pos_] == '.' ||
                                              ((src_[pos_] == 'p' || src_[pos_] == 'P')) ||
                                              ((src_[pos_] == '+' || src_[pos_] == '-') &&
                                               (src_[pos_ - 1] == 'p' || src_[pos_ - 1] == 'P'))))
                    ++pos_;
            } else {
                while (pos_ < src_.size() && (std::isdigit((unsigned char)src_[pos_]) || src_[pos_] == '.')) ++pos_;
                if (pos_ < src_.size() && (src_[pos_] == 'e' || src_[pos_] == 'E')) {
                    ++pos_;
                    if (pos_ < src_.size() && (src_[pos_] == '+' || src_[pos_] == '-')) ++pos_;
                    while (pos_ < src_.size() && std::isdigit((unsigned char)src_[pos_])) ++pos_;
                }
            }
            if (pos_ < src_.size() && (std::isalnum((unsigned char)src_[pos_]) || src_[pos_] == '_'))
                error("malformed number near '" + src_.substr(b, pos_ - b + 1) + "'");
            std::string t = src_.substr(b, pos_ - b);
            char* end = nullptr;
            errno = 0;
            double v = std::strtod(t.c_str(), &end);
            if (!end || *end) error("malformed number '" + t + "'");
            tok_.kind = T_NUMBER;
            tok_.num = v;
            tok_.text = t;
            return;
        }
        if (c == '\'' || c == '"') {
            ++pos_;
            std::string out;
            for (;;) {
                if (pos_ >= src_.size() || src_[pos_] == '\n') error("unfinished string", line_);
                char d = src_[pos_++];
                if (d == c) break;
                if (d == '\\') {
                    if (pos_ >= src_.size()) error("unfinished string", line_);
                    char e = src_[pos_++];
                    switch (e) {
                    case 'n': out += '\n'; break;
                    case 't': out += '\t'; break;
                    case '\\': out += '\\'; break;
                    case '\'': out += '\''; break;
                    case '"': out += '"'; break;
                    default: error(std::string("unsupported escape '\\") + e + "' in a string", line_);
                    }
                } else {
                    out += d;
                }
            }
            tok_.kind = T_STRING;
            tok_.text = out;
            return;
        }
        static const char* two[] = {"==", "~=", "<=", ">=", ".."};
        for (const char* op : two)
            if (src_.compare(pos_, 2, op) == 0) {
                tok_.kind = T_OP;
                tok_.text = op;
                pos_ += 2;
                return;
            }
        tok_.kind = T_OP;
        tok_.text = std::string(1, c);
        ++pos_;
    }

    bool isOp(const char* op) const { return tok_.kind == T_OP && tok_.text == op; }
    bool isName(const char* n) const { return tok_.kind == T_NAME && tok_.text == n; }
    void expectOp(const char* op) {
        if (!isOp(op)) error(std::string("'") + op + "' expected near '" + describe() + "'");
        next();
    }
    std::string describe() const { return tok_.kind == T_EOF ? "<eof>" : tok_.text; }

    static bool reserved(const std::string& w) {
        static const char* kw[] = {"and", "break", "do", "else", "elseif", "end", "false", "for", "function",
                                   "goto", "if", "in", "local", "nil", "not", "or", "repeat", "return", "then",
                                   "true", "until", "while"};
        for (const char* k : kw)
            if (w == k) return true;
        return false;
    }

    static Value number(double v) {
        Value r;
        r.kind = Value::NUMBER;
        r.n = v;
        return r;
    }

    // a table key from a value (number keys with an integer value are integers)
    struct Key {
        bool isNum;
        long long i;
        std::string s;
    };
    Key keyOf(const Value& v, int line) const {
        if (v.kind == Value::STRING) return {false, 0, v.s};
        if (v.kind == Value::NUMBER) {
            if (std::floor(v.n) == v.n && std::fabs(v.n) < 9.0e15) return {true, (long long)v.n, ""};
            error("table keys that are not integers or strings are not supported", line);
        }
        error("table key must be a number or a string", line);
    }
    static Value get(const Table& t, const Key& k) {
        if (k.isNum) {
            auto it = t.arr.find(k.i);
            return it == t.arr.end() ? Value() : it->second;
        }
        auto it = t.hash.find(k.s);
        return it == t.hash.end() ? Value() : it->second;
    }
    static void set(Table& t, const Key& k, const Value& v) {
        if (k.isNum) {
            if (v.kind == Value::NIL) t.arr.erase(k.i);
            else t.arr[k.i] = v;
        } else {
            if (v.kind == Value::NIL) t.hash.erase(k.s);
            else t.hash[k.s] = v;
        }
    }

    void statement() {
        if (isOp(";")) { next(); return; }
        const int line = tok_.line;
        if (tok_.kind != T_NAME || reserved(tok_.text))
            error("only assignments of values can be read here, not '" + describe() + "'");
        std::string root = tok_.text;
        next();
        std::vector<Key> path;
        for (;;) {
            if (isOp(".")) {
                next();
                if (tok_.kind != T_NAME) error("name expected after '.'");
                path.push_back({false, 0, tok_.text});
                next();
            } else if (isOp("[")) {
                next();
                Value k = expr();
                expectOp("]");
                path.push_back(keyOf(k, line));
            } else {
                break;
            }
        }
        if (!isOp("=")) {
            if (isOp("(") || tok_.kind == T_STRING || isOp("{") || isOp(":"))
                error("function calls cannot be evaluated without a Lua interpreter ('" + root + "')", line);
            error("'=' expected after '" + root + "'", line);
        }
        next();
        Value v = expr();
        if (isOp(",")) error("multiple assignment is not supported", line);
        if (path.empty()) {
            if (v.kind == Value::NIL) globals.erase(root);
            else globals[root] = v;
            return;
        }
        auto it = globals.find(root);
        if (it == globals.end() || it->second.kind != Value::TABLE)
            error("attempt to index '" + root + "', which is not a table", line);
        std::shared_ptr<Table> t = it->second.t;
        for (size_t i = 0; i + 1 < path.size(); ++i) {
            Value inner = get(*t, path[i]);
            if (inner.kind != Value::TABLE) error("attempt to index a field that is not a table", line);
            t = inner.t;
        }
        set(*t, path.back(), v);
    }

    // precedence (low to high): + -, * / %, unary -, ^ (right associative)
    Value expr() {
        if (isName("and") || isName("or") || isName("not"))
            error("logical operators are not supported");
        Value a = term();
        while (isOp("+") || isOp("-")) {
            bool add = tok_.text == "+";
            int line = tok_.line;
            next();
            Value b = term();
            a = number(add ? num(a, line) + num(b, line) : num(a, line) - num(b, line));
        }
        rejectOther();
        return a;
    }
    void rejectOther() {
        if (isOp("..")) error("string concatenation is not supported");
        if (isOp("==") || isOp("~=") || isOp("<") || isOp(">") || isOp("<=") || isOp(">="))
            error("comparisons are not supported");
        if (isName("and") || isName("or")) error("logical operators are not supported");
    }
    Value term() {
        Value a = unary();
        while (isOp("*") || isOp("/") || isOp("%")) {
            char op = tok_.text[0];
            int line = tok_.line;
            next();
            Value b = unary();
            double x = num(a, line), y = num(b, line);
            a = number(op == '*' ? x * y : op == '/' ? x / y : x - std::floor(x / y) * y);
        }
        return a;
    }
    Value unary() {
        if (isOp("-")) {
            int line = tok_.line;
            next();
            Value v = unary();
            return number(-num(v, line));
        }
        if (isName("not")) error("logical operators are not supported");
        if (isOp("#")) error("the length operator is not supported");
        return power();
    }
    Value power() {
        Value a = primary();
        if (isOp("^")) {
            int line = tok_.line;
            next();
            Value b = unary();   // right associative, binds tighter than a unary minus on its left
            return number(std::pow(num(a, line), num(b, line)));
        }
        return a;
    }
    double num(const Value& v, int line) const {
        if (v.kind != Value::NUMBER) error("arithmetic on a value that is not a number", line);
        return v.n;
    }
    Value primary() {
        const int line = tok_.line;
        if (tok_.kind == T_NUMBER) { double v = tok_.num; next(); return number(v); }
        if (tok_.kind == T_STRING) {
            Value r;
            r.kind = Value::STRING;
            r.s = tok_.text;
            next();
            if (tok_.kind == T_STRING || isOp("(")) error("function calls are not supported", line);
            return r;
        }
        if (isName("true") || isName("false")) {
            Value r;
            r.kind = Value::BOOL;
            r.b = tok_.text == "true";
            next();
            return r;
        }
        if (isName("nil")) { next(); return Value(); }
        if (isName("function")) error("functions cannot be evaluated without a Lua interpreter");
        if (isOp("{")) return table();
        if (isOp("(")) {
            next();
            Value v = expr();
            expectOp(")");
            return v;
        }
        if (tok_.kind == T_NAME && !reserved(tok_.text)) {
            std::string name = tok_.text;
            next();
            auto it = globals.find(name);
            Value v = it == globals.end() ? Value() : it->second;
            for (;;) {
                if (isOp(".") || isOp("[")) {
                    Key k;
                    if (isOp(".")) {
                        next();
                        if (tok_.kind != T_NAME) error("name expected after '.'");
                        k = {false, 0, tok_.text};
                        next();
                    } else {
                        next();
                        Value kv = expr();
                        expectOp("]");
                        k = keyOf(kv, line);
                    }
                    if (v.kind != Value::TABLE) error("attempt to index '" + name + "', which is not a table", line);
                    v = get(*v.t, k);
                } else if (isOp("(") || isOp(":") || tok_.kind == T_STRING || isOp("{")) {
                    error("function calls cannot be evaluated without a Lua interpreter ('" + name + "')", line);
                } else {
                    break;
                }
            }
            return v;
        }
        error("unexpected '" + describe() + "'");
    }
    Value table() {
        const int line = tok_.line;
        expectOp("{");
        auto t = std::make_shared<Table>();
        long long nextIndex = 1;
        while (!isOp("}")) {
            if (isOp("[")) {
                next();
                Value k = expr();
                expectOp("]");
                expectOp("=");
                set(*t, keyOf(k, line), expr());
            } else if (tok_.kind == T_NAME && !reserved(tok_.text)) {
                // Name = expr, or an expression that starts with a name
                size_t savePos = pos_;
                int saveLine = line_;
                Tok save = tok_;
                next();
                if (isOp("=")) {
                    next();
                    set(*t, {false, 0, save.text}, expr());
                } else {
                    pos_ = savePos;
                    line_ = saveLine;
                    tok_ = save;
                    set(*t, {true, nextIndex++, ""}, expr());
                }
            } else {
                set(*t, {true, nextIndex++, ""}, expr());
            }
            if (isOp(",") || isOp(";")) next();
            else if (!isOp("}")) error("'}' expected (to close '{' at line " + std::to_string(line) + ")");
        }
        next();
        Value r;
        r.kind = Value::TABLE;
        r.t = t;
        return r;
    }
};

[[noreturn]] void bad(int status, const std::string& msg) { throw ParseError{status, msg}; }

const Value* global(const Reader& r, const char* key) {
    auto it = r.globals.find(key);
    return it == r.globals.end() ? nullptr : &it->second;
}

std::string str(const Value& v, const char* key) {
    if (v.kind != Value::STRING) bad(HGPU_ERR_CONFIG, std::string(key) + " must be a string");
    return v.s;
}
double numv(const Value& v, const char* key) {
    if (v.kind == Value::NUMBER) return v.n;
    if (v.kind == Value::STRING) {
        // LuaCxx's numeric read of a string goes through Lua's coercion (tonumber)
        char* end = nullptr;
        double d = std::strtod(v.s.c_str(), &end);
        if (end && end != v.s.c_str() && *end == 0) return d;
    }
    bad(HGPU_ERR_CONFIG, std::string(key) + " must be a number");
}
// Lua truthiness for the reference's bool reads: only nil and false are false
bool truthy(const Value& v) { return !(v.kind == Value::NIL || (v.kind == Value::BOOL && !v.b)); }
int intv(const Value& v, const char* key) {
    double d = numv(v, key);
    if (!(std::floor(d) == d) || std::fabs(d) > 2147483647.)
        bad(HGPU_ERR_CONFIG, std::string(key) + " must be an integer");
    return (int)d;
}

int indexOf(const std::string& name, const char* const* names, int n) {
    for (int i = 0; i < n; ++i)
        if (name == names[i]) return i;
    return -1;
}

const char* const kSolvers[] = {"EulerRoe", "EulerHLLC", "EulerHLL"};
const char* const kIntegrators[] = {"ForwardEuler", "RungeKutta2", "RungeKutta2Heun", "RungeKutta2Ralston",
                                    "RungeKutta3", "RungeKutta4", "RungeKutta4_3_8thsRule", "RungeKutta2TVD",
                                    "RungeKutta2NonTVD", "RungeKutta3TVD", "RungeKutta4TVD", "RungeKutta4NonTVD"};
const char* const kLimiters[] = {"DonorCell", "LaxWendroff", "BeamWarming", "Fromm", "CHARM", "HCUS", "HQUICK",
                                 "Koren", "MinMod", "Oshker", "Ospre", "Smart", "Sweby", "UMIST", "VanAlbada1",
                                 "VanAlbada2", "VanLeer", "MonotizedCentral", "Superbee", "BarthJespersen"};
const char* const kBoundaries[] = {"PERIODIC", "MIRROR", "FREEFLOW"};

void apply(const Reader& r, hgpu_config* cfg) {
    const Value* v;
    // solver: HydroGPUApp.cpp:330-348 (Euler solvers of the registry, :90-118)
    v = global(r, "solverName");
    if (!v) bad(HGPU_ERR_UNSUPPORTED, "solverName not set: the reference's default, EulerBurgers, is not provided");
    {
        std::string s = str(*v, "solverName");
        int k = indexOf(s, kSolvers, 3);
        if (k < 0) bad(s == "EulerBurgers" ? HGPU_ERR_UNSUPPORTED : HGPU_ERR_CONFIG, "unknown solver " + s);
        cfg->solver = k;
    }
    // integrator: Solver.cpp:178-204
    if ((v = global(r, "integratorName"))) {
        std::string s = str(*v, "integratorName");
        int k = indexOf(s, kIntegrators, HGPU_NUM_INTEGRATORS);
        if (k < 0) bad(s == "BackwardEulerConjugateGradient" ? HGPU_ERR_UNSUPPORTED : HGPU_ERR_CONFIG,
                       "failed to find integrator named " + s);
        cfg->integrator = k;
    }
    // slope limiter: the key the solver reads (Solver.cpp:285-287); slopeLimiterName is not it
    if ((v = global(r, "slopeLimiter"))) {
        std::string s = str(*v, "slopeLimiter");
        int k = indexOf(s, kLimiters, HGPU_NUM_LIMITERS);
        if (k < 0) bad(HGPU_ERR_CONFIG, "unknown slope limiter " + s);
        cfg->limiter = k;
    }
    // size / xmin / xmax: HydroGPUApp.cpp:166-170 (size[i+1] for i = 0..2; absent entries are 1)
    if ((v = global(r, "size"))) {
        if (v->kind != Value::TABLE) bad(HGPU_ERR_CONFIG, "size must be a table");
        for (int i = 0; i < 3; ++i) {
            auto it = v->t->arr.find(i + 1);
            cfg->size[i] = it == v->t->arr.end() ? 1 : intv(it->second, "size[i]");
        }
    }
    const char* bounds[2] = {"xmin", "xmax"};
    for (int m = 0; m < 2; ++m) {
        if (!(v = global(r, bounds[m]))) continue;
        if (v->kind != Value::TABLE) bad(HGPU_ERR_CONFIG, std::string(bounds[m]) + " must be a table");
        for (int i = 0; i < 3; ++i) {
            auto it = v->t->arr.find(i + 1);
            if (it != v->t->arr.end()) (m ? cfg->xmax : cfg->xmin)[i] = numv(it->second, bounds[m]);
        }
    }
    // boundaryMethods: HydroGPUApp.cpp:172-181 (names), 495-511 (lookup; "NONE" is -1)
    if ((v = global(r, "boundaryMethods"))) {
        if (v->kind != Value::TABLE) bad(HGPU_ERR_CONFIG, "boundaryMethods must be a table");
        for (int i = 0; i < 3; ++i) {
            auto it = v->t->arr.find(i + 1);
            if (it == v->t->arr.end() || it->second.kind != Value::TABLE) continue;
            const char* mm[2] = {"min", "max"};
            for (int m = 0; m < 2; ++m) {
                auto jt = it->second.t->hash.find(mm[m]);
                if (jt == it->second.t->hash.end()) continue;
                std::string s = str(jt->second, "boundaryMethods[i].min/max");
                if (s.empty()) continue;
                int k = indexOf(s, kBoundaries, 3);
                if (k < 0 && s != "NONE") bad(HGPU_ERR_CONFIG, "couldn't interpret boundary method " + s);
                cfg->boundary[i][m] = k < 0 ? HGPU_BOUNDARY_NONE : k;
            }
        }
    }
    // HydroGPUApp.cpp:204-208
    if ((v = global(r, "cfl"))) cfg->cfl = (float)numv(*v, "cfl");
    if ((v = global(r, "useFixedDT"))) cfg->use_fixed_dt = truthy(*v) ? 1 : 0;
    if ((v = global(r, "fixedDT"))) cfg->fixed_dt = numv(*v, "fixedDT");
    if ((v = global(r, "useGravity"))) cfg->use_gravity = truthy(*v) ? 1 : 0;
    if ((v = global(r, "gaussSeidelMaxIter"))) cfg->gauss_seidel_max_iter = intv(*v, "gaussSeidelMaxIter");
    // defs: Solver.cpp:289-299 (each becomes #define KEY ((real)value))
    if ((v = global(r, "defs"))) {
        if (v->kind != Value::TABLE) bad(HGPU_ERR_CONFIG, "defs must be a table");
        auto g = v->t->hash.find("idealGas_heatCapacityRatio");
        if (g != v->t->hash.end()) cfg->gamma = numv(g->second, "defs.idealGas_heatCapacityRatio");
        auto G = v->t->hash.find("selfGrav_gravitationalConstant");
        if (G != v->t->hash.end()) cfg->gravitational_constant = numv(G->second, "defs.selfGrav_gravitationalConstant");
    }
}

int fromText(const std::string& text, hgpu_config* cfg) {
    hgpu_config out;
    hgpu_config_default(&out);
    try {
        Reader r(text);
        r.run();
        apply(r, &out);
    } catch (const ParseError& e) {
        hgpu::setLastError(e.msg);
        return e.status;
    } catch (const std::bad_alloc&) {
        hgpu::setLastError("host allocation failed");
        return HGPU_ERR_NOMEM;
    }
    *cfg = out;
    return HGPU_OK;
}

}  // namespace

extern "C" {

int hgpu_config_from_string(const char* text, hgpu_config* cfg) {
    if (!text || !cfg) {
        hgpu::setLastError("null argument");
        return HGPU_ERR_ARG;
    }
    return fromText(text, cfg);
}

int hgpu_config_from_file(const char* path, hgpu_config* cfg) {
    if (!path || !cfg) {
        hgpu::setLastError("null argument");
        return HGPU_ERR_ARG;
    }
    FILE* f = std::fopen(path, "rb");
    if (!f) {
        hgpu::setLastError(std::string("cannot open config file ") + path);
        return HGPU_ERR_ARG;
    }
    std::string text;
    char buf[4096];
    size_t n;
    while ((n = std::fread(buf, 1, sizeof buf, f)) > 0) text.append(buf, n);
    std::fclose(f);
    if (text.find('\0') != std::string::npos) {
        hgpu::setLastError(std::string("config file contains a NUL byte: ") + path);
        return HGPU_ERR_CONFIG;
    }
    return fromText(text, cfg);
}

}  // extern "C"
