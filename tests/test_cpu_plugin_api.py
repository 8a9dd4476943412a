"""The C++ plugin layer (include/gb_hybrid_pt.h) keeps the reference's
gi_algorithm registry semantics (gi_algorithm.h:26-49): duplicate names
throw std::logic_error, select() of an unknown name throws
std::runtime_error, select() activates once, list() keeps registration
order, and the knob defaults print the reference's messages."""
import subprocess
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent

PROG = r'''
#include "gb_hybrid_pt.h"
#include <cstdio>
struct counting : gb::gi_algorithm {
    int activations = 0, computes = 0;
    explicit counting(const std::string& n) : gi_algorithm(n) {}
    void activate(gb::rt_set* s) override { ++activations; gi_algorithm::activate(s); }
    void compute() override { ++computes; }
};
int main() {
    counting a("a"), b("b");
    int fails = 0;
    try { counting dup("a"); ++fails; } catch (const std::logic_error&) {}
    try { gb::gi_algorithm::select("nope"); ++fails; } catch (const std::runtime_error&) {}
    gb::gi_algorithm::select("b");
    gb::gi_algorithm::select("b");
    if (b.activations != 1 || gb::gi_algorithm::selected() != &b) ++fails;
    if (gb::gi_algorithm::get("a") != &a || gb::gi_algorithm::get("zz") != nullptr) ++fails;
    auto l = gb::gi_algorithm::list();
    if (l.size() != 2 || l.front() != "a") ++fails;
    b.update();
    if (b.computes != 1) ++fails;
    a.path_samples(4);
    std::printf("%d\n", fails);
    return fails;
}
'''


def test_registry_semantics(tmp_path, lib_path):
    src = tmp_path / "t.cpp"
    src.write_text(PROG)
    exe = tmp_path / "t"
    subprocess.run(["g++", "-std=c++17", "-I", str(ROOT / "include"), str(src), "-o", str(exe),
                    "-L", str(lib_path.parent), "-lgbpt", f"-Wl,-rpath,{lib_path.parent}"], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "does not know about path samples" in r.stderr
