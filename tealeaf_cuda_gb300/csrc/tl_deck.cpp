// tl_deck.cpp -- the tea.in reader: the keyword parser of parse.f90 (line
// clean-up, *tea ... *endtea section, blank-separated words, `\` and value
// wrap across lines, I7 / E27.20 conversions) and the keyword table and
// defaults of read_input.f90:38-327, plus the flags this implementation adds
// (tl_precision, tl_inner_eps, cuda_device).
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/tealeaf_capi.h"

namespace {

struct DeckError {
    int code;
    std::string msg;
};

class Deck {
  public:
    explicit Deck(const char *text) {
        std::string cur;
        for (const char *q = text; *q; ++q) {
            if (*q == '\n') {
                raw_.push_back(cur);
                cur.clear();
            } else {
                cur.push_back(*q);
            }
        }
        if (!cur.empty()) raw_.push_back(cur);
    }

    void rewind() {
        pos_ = 0;
        here_.clear();
        line_.clear();
    }

    // parse_getline (parse.f90:119-237) for the "*tea" section
    bool next_line() {
        while (pos_ < raw_.size()) {
            std::string l = raw_[pos_++];
            if (l.size() > 100) l.resize(100);  // FMT='(a100)'
            for (char &ch : l) {
                const unsigned char u = (unsigned char)ch;
                if (u < 32 || u > 128) ch = ' ';
            }
            size_t b = l.find_first_not_of(' ');
            l = b == std::string::npos ? std::string() : l.substr(b);
            size_t cut = l.find('!');
            if (cut != std::string::npos) l.resize(cut);
            cut = l.find(';');
            if (cut != std::string::npos) l.resize(cut);
            while (!l.empty() && l.back() == ' ') l.pop_back();
            for (char &ch : l) {
                ch = (char)std::tolower((unsigned char)ch);
                if (ch == '=' || ch == ',') ch = ' ';
            }
            if (!l.empty() && l[0] == '*') {
                std::string nugget = l.substr(0, l.find(' '));
                if (nugget.compare(1, 3, "end") == 0) {
                    const std::string closing = "*" + nugget.substr(4);
                    const size_t last = here_.rfind('*');
                    if (last != std::string::npos && here_.substr(last) == closing) {
                        const bool was_mask = here_ == "*tea";
                        here_.resize(last);
                        if (was_mask) {
                            pos_ = raw_.size();
                            return false;
                        }
                    }
                } else {
                    here_ += nugget;
                }
                continue;
            }
            if (here_ == "*tea" && !l.empty()) {
                line_ = l;
                return true;
            }
        }
        return false;
    }

    // parse_getword (parse.f90:239-265)
    std::string word(bool wrap) {
        for (;;) {
            size_t b = line_.find_first_not_of(' ');
            if (b == std::string::npos) line_.clear();
            else line_ = line_.substr(b);
            size_t e = line_.find(' ');
            std::string w = line_.substr(0, e);
            if (w == "\\" || (w.empty() && wrap)) {
                if (!next_line()) return std::string();
                continue;
            }
            line_ = e == std::string::npos ? std::string() : line_.substr(e);
            return w;
        }
    }

    int ival(bool wrap = true) {
        std::string w = word(wrap);
        std::string s = w.substr(0, 7);  // FMT="(I7)"
        char *end = nullptr;
        long v = std::strtol(s.c_str(), &end, 10);
        if (s.empty() || *end != '\0') throw DeckError{TL_ERR_DECK, "Error attempting to convert to integer:" + w};
        return (int)v;
    }

    double rval() {
        std::string w = word(true);
        std::string s = w;
        for (char &ch : s)
            if (ch == 'd') ch = 'e';
        char *end = nullptr;
        double v = std::strtod(s.c_str(), &end);
        if (s.empty() || end == s.c_str() || (*end != '\0' && w.find('.') != std::string::npos))
            throw DeckError{TL_ERR_DECK, "Error attempting to convert to real:" + w};
        return v;
    }

  private:
    std::vector<std::string> raw_;
    size_t pos_ = 0;
    std::string here_;
    std::string line_;
};

void defaults(tl_config_t *c) {
    std::memset(c, 0, sizeof *c);
    c->xmin = 0.0;
    c->ymin = 0.0;
    c->xmax = 100.0;
    c->ymax = 100.0;
    c->x_cells = 10;
    c->y_cells = 10;
    c->end_time = 10.0;
    c->end_step = 640000;  // g_ibig
    c->summary_frequency = 10;
    c->dtinit = 0.1;
    c->max_iters = 1000;
    c->eps = 1.0e-10;
    c->coefficient = TL_COEF_CONDUCTIVITY;
    c->ch_cg_presteps = 25;
    c->ch_cg_epslim = 1.0;
    c->precond = TL_PREC_NONE;
    c->ppcg_inner_steps = -1;
    c->solver = TL_SOLVER_JACOBI;
    c->halo_depth = 1;
    c->precision = TL_PRECISION_FP64;
    c->inner_eps = 1.0e-6;
}

void parse(const char *text, tl_config_t *c) {
    defaults(c);
    Deck d(text);
    // number of states (read_input.f90:94-106)
    int state_max = 0;
    while (d.next_line()) {
        for (std::string w = d.word(false); !w.empty(); w = d.word(false))
            if (w == "state") {
                int s = d.ival();
                if (s > state_max) state_max = s;
                break;
            }
    }
    if (state_max < 1) throw DeckError{TL_ERR_DECK, "No states defined."};
    if (state_max > TL_MAX_STATES) throw DeckError{TL_ERR_DECK, "too many states"};
    c->nstates = state_max;
    std::vector<bool> defined(state_max, false);
    d.rewind();
    while (d.next_line()) {
        for (std::string w = d.word(false); !w.empty(); w = d.word(false)) {
            if (w == "initial_timestep") c->dtinit = d.rval();
            else if (w == "end_time") c->end_time = d.rval();
            else if (w == "end_step") c->end_step = d.ival();
            else if (w == "xmin") c->xmin = d.rval();
            else if (w == "xmax") c->xmax = d.rval();
            else if (w == "ymin") c->ymin = d.rval();
            else if (w == "ymax") c->ymax = d.rval();
            else if (w == "x_cells") c->x_cells = d.ival();
            else if (w == "y_cells") c->y_cells = d.ival();
            else if (w == "visit_frequency") (void)d.ival();
            else if (w == "summary_frequency") c->summary_frequency = d.ival();
            else if (w == "tl_ch_cg_presteps") c->ch_cg_presteps = d.ival();
            else if (w == "tl_ppcg_inner_steps") c->ppcg_inner_steps = d.ival();
            else if (w == "tl_ch_cg_epslim") c->ch_cg_epslim = d.rval();
            else if (w == "tl_check_result") c->check_result = 1;
            else if (w == "tl_preconditioner_type") {
                for (std::string v = d.word(false); !v.empty(); v = d.word(false)) {
                    if (v == "none") c->precond = TL_PREC_NONE;
                    else if (v == "jac_diag") c->precond = TL_PREC_JAC_DIAG;
                    else if (v == "jac_block") c->precond = TL_PREC_JAC_BLOCK;
                    else throw DeckError{TL_ERR_DECK, "Invalid preconditioner type specified: " + v};
                }
            }
            else if (w == "use_cuda_kernels") {}
            else if (w == "verbose_on") c->verbose = 1;
            else if (w == "tl_use_jacobi") c->solver = TL_SOLVER_JACOBI;
            else if (w == "tl_use_cg") c->solver = TL_SOLVER_CG;
            else if (w == "tl_use_ppcg") c->solver = TL_SOLVER_PPCG;
            else if (w == "tl_use_chebyshev") c->solver = TL_SOLVER_CHEBYSHEV;
            else if (w == "reflective_boundary") c->reflective_boundary = 1;
            else if (w == "profiler_on") c->profiler_on = 1;
            else if (w == "halo_depth") {
                c->halo_depth = d.ival();
                if (c->halo_depth < 1) throw DeckError{TL_ERR_DECK, "Invalid halo exchange depth specified"};
            }
            else if (w == "tl_max_iters") c->max_iters = d.ival();
            else if (w == "tl_eps") c->eps = d.rval();
            else if (w == "tl_coefficient_density") c->coefficient = TL_COEF_CONDUCTIVITY;
            else if (w == "tl_coefficient_inverse_density") c->coefficient = TL_COEF_RECIP_CONDUCTIVITY;
            else if (w == "test_problem") c->test_problem = d.ival();
            else if (w == "cuda_device") c->cuda_device = d.ival();
            else if (w == "tl_precision") {
                std::string v = d.word(true);
                if (v == "fp64") c->precision = TL_PRECISION_FP64;
                else if (v == "mixed") c->precision = TL_PRECISION_MIXED;
                else throw DeckError{TL_ERR_DECK, "Invalid tl_precision: " + v};
            }
            else if (w == "tl_inner_eps") c->inner_eps = d.rval();
            else if (w == "tl_warm_start") {
                std::string v = d.word(true);
                if (v == "none") c->warm_start = TL_WARM_NONE;
                else if (v == "prev") c->warm_start = TL_WARM_PREV;
                else if (v == "learned") c->warm_start = TL_WARM_LEARNED;
                else throw DeckError{TL_ERR_DECK, "Invalid tl_warm_start: " + v};
            }
            else if (w == "state") {
                const int s = d.ival();
                if (s < 1 || s > state_max) throw DeckError{TL_ERR_DECK, "Invalid state number"};
                if (defined[s - 1]) throw DeckError{TL_ERR_DECK, "State defined twice."};
                defined[s - 1] = true;
                tl_state_t &st = c->states[s - 1];
                for (std::string k = d.word(false); !k.empty(); k = d.word(false)) {
                    if (k == "xmin") st.xmin = d.rval();
                    else if (k == "ymin") st.ymin = d.rval();
                    else if (k == "xmax") st.xmax = d.rval();
                    else if (k == "ymax") st.ymax = d.rval();
                    else if (k == "radius") st.radius = d.rval();
                    else if (k == "density") st.density = d.rval();
                    else if (k == "energy") st.energy = d.rval();
                    else if (k == "geometry") {
                        std::string g = d.word(true);
                        if (g == "rectangle") st.geometry = TL_GEOM_RECTANGLE;
                        else if (g == "circle") st.geometry = TL_GEOM_CIRCLE;
                        else if (g == "point") st.geometry = TL_GEOM_POINT;
                    }
                }
            }
        }
    }
    // read_input.f90:294-297 (REAL(4) arithmetic)
    if (c->ppcg_inner_steps == -1) {
        const float cells = (float)(c->x_cells * c->y_cells);
        c->ppcg_inner_steps = 4 * (int)std::sqrt(std::sqrt(cells));
    }
    if (c->halo_depth > 1 && c->precond == TL_PREC_JAC_BLOCK && c->solver == TL_SOLVER_PPCG)
        throw DeckError{TL_ERR_DECK, "Unable to use nonstandard halo depth with block jacobi preconditioner"};
    // read_input.f90:320-327
    const double dx = (c->xmax - c->xmin) / (double)(float)c->x_cells;
    const double dy = (c->ymax - c->ymin) / (double)(float)c->y_cells;
    for (int n = 1; n < c->nstates; ++n) {
        c->states[n].xmin += dx / 100.0;
        c->states[n].ymin += dy / 100.0;
        c->states[n].xmax -= dx / 100.0;
        c->states[n].ymax -= dy / 100.0;
    }
}

}  // namespace

extern "C" int tl_parse_deck(const char *deck_text, tl_config_t *cfg, char *err, int errlen) {
    if (!deck_text || !cfg) return TL_ERR_ARG;
    try {
        parse(deck_text, cfg);
    } catch (const DeckError &e) {
        if (err && errlen > 0) std::snprintf(err, (size_t)errlen, "%s", e.msg.c_str());
        return e.code;
    }
    if (err && errlen > 0) err[0] = '\0';
    return TL_OK;
}
