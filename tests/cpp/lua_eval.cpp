// Runs a Lua chunk through shoccs_gb300/app/lua_subset.hpp and prints the global table
// `result` flattened, one "path<TAB>type<TAB>value" line per leaf, for tests/test_cli.py.
// A Lua error prints "error<TAB>message" and exits 1.
#include "lua_subset.hpp"

#include <cstdio>
#include <string>

namespace
{
void dump(const std::string& path, const ccs::lua::value& v)
{
    using namespace ccs::lua;
    if (auto t = v.tbl()) {
        for (const auto& [k, x] : t->ints) dump(path + "[" + std::to_string(k) + "]", x);
        for (const auto& [k, x] : t->reals) dump(path + "[" + to_display(value{k}) + "]", x);
        for (const auto& [k, x] : t->strs) dump(path + "." + k, x);
        return;
    }
    if (auto d = v.number()) {
        std::printf("%s\tnumber\t%.17g\n", path.c_str(), *d);
        return;
    }
    std::printf("%s\t%s\t%s\n", path.c_str(), v.type_name(), to_display(v).c_str());
}
} // namespace

int main(int argc, char** argv)
{
    if (argc < 2) return 2;
    ccs::lua::state L;
    try {
        L.script_file(argv[1]);
        for (int i = 2; i < argc; i++) L.script(argv[i], "script");
    } catch (const ccs::lua::error& e) {
        std::printf("error\t%s\n", e.what());
        return 1;
    }
    dump("result", L.get("result"));
    return 0;
}
