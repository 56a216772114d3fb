// Link check of the reference-side binding (test infrastructure): a program
// made of the reference's own objects (built by build_ref.py) and the
// GpuTransporter of include/abeille_gb300_transporter.hpp, linked with
// libabeille_gb300.so.
//
//   adapter_check DECK.yaml
//
// Reads the deck natively (abx_deck_read) and prints what it holds, then
// constructs a GpuTransporter over the reference's Tallies.  Without a GPU
// the construction fails in abx_create and the reference's fatal_error ends
// the program with status 1 and the engine's reason; with one it prints
// "context created".
#include <abeille_gb300_transporter.hpp>

#include <cstdio>
#include <fstream>
#include <memory>
#include <sstream>
#include <string>

int main(int argc, char** argv) {
  if (argc != 2) {
    std::fprintf(stderr, "usage: adapter_check DECK.yaml\n");
    return 2;
  }
  std::ifstream f(argv[1]);
  std::stringstream b;
  b << f.rdbuf();
  const std::string text = b.str();
  abx_deck* deck = nullptr;
  const abx_problem* p = nullptr;
  if (abx_deck_read(text.c_str(), ABX_PREC_FP64, &deck, &p) != ABX_OK) {
    std::printf("deck refused: %s\n", abx_last_error_string());
    return 3;
  }
  std::printf("deck: %d surfaces, %d cells, %d universes, %d materials, %d tallies, %d sources, %d groups\n",
              p->n_surfaces, p->n_cells, p->n_universes, p->n_materials, p->n_tallies, p->n_sources,
              p->settings.ngroups);
  std::fflush(stdout);
  abx_deck_free(deck);
  auto tallies = std::make_shared<Tallies>(1.0);
  GpuTransporter t(tallies, text, ABX_PREC_FP64);
  std::printf("context created\n");
  return 0;
}
