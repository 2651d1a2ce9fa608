// LEMS expression parser used ONLY to link the reference EDEN oracle binary.
//
// Test infrastructure: this file is compiled into oracle/_ref/eden, the
// reference's own CPU simulator built from its unmodified sources, which is
// the parity checker for the GPU path.  It is never linked into the product.
//
// The reference generates its expression parser with flex + bison
// (eden/neuroml/LEMS_Expr.lex, eden/neuroml/LEMS_Expr.y); neither tool is
// installed here, so this is a hand-written recursive-descent parser that
// produces the same TermTable trees.  It follows:
//   * tokens:      LEMS_Expr.lex:31-96 (numbers, operators, dotted and
//                  symbolic comparison / logic words, function names, "H",
//                  identifiers; keywords win only on an exact identifier
//                  match, as flex's longest-match rule gives)
//   * precedence:  LEMS_Expr.y:86-98, lowest first: or, and, == !=, >= <=,
//                  + -, * /, ^ (right assoc), functions, not, unary minus.
//                  Unary minus binds tighter than ^ ( -a^b == (-a)^b ).
//   * productions: LEMS_Expr.y:102-160 (anyexpr, numexpr, binexpr,
//                  num_function, symexpr)
// Its header is the reference's eden/neuroml/LEMS_Expr.h (include path).
#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "LEMS_Expr.h"

namespace {

enum Tok {
    T_END, T_NUM, T_SYM, T_PLUS, T_MINUS, T_TIMES, T_DIV, T_POW, T_LP, T_RP,
    T_LEQ, T_GEQ, T_LT, T_GT, T_EQ, T_NEQ, T_AND, T_OR, T_NOT,
    T_FUNC, T_BAD
};

struct Token {
    Tok kind;
    double value = 0;
    std::string text;
    Term::Type func = Term::NONE;  // for T_FUNC
    int pos = 0;
};

struct Keyword { const char *word; Tok kind; Term::Type func; };

const Keyword kWords[] = {
    {"and", T_AND, Term::NONE},     {"or", T_OR, Term::NONE},
    {"not", T_NOT, Term::NONE},     {"abs", T_FUNC, Term::ABS},
    {"sqrt", T_FUNC, Term::SQRT},   {"sin", T_FUNC, Term::SIN},
    {"cos", T_FUNC, Term::COS},     {"tan", T_FUNC, Term::TAN},
    {"sinh", T_FUNC, Term::SINH},   {"cosh", T_FUNC, Term::COSH},
    {"tanh", T_FUNC, Term::TANH},   {"exp", T_FUNC, Term::EXP},
    {"log10", T_FUNC, Term::LOG10}, {"log", T_FUNC, Term::LN},
    {"ln", T_FUNC, Term::LN},       {"ceil", T_FUNC, Term::CEIL},
    {"floor", T_FUNC, Term::FLOOR}, {"int", T_FUNC, Term::INT},
    {"random", T_FUNC, Term::RANDOM}, {"H", T_FUNC, Term::HFUNC},
};

const struct { const char *text; Tok kind; } kDotted[] = {
    {".leq.", T_LEQ}, {".geq.", T_GEQ}, {".neq.", T_NEQ}, {".and.", T_AND},
    {".not.", T_NOT}, {".lt.", T_LT},   {".gt.", T_GT},   {".eq.", T_EQ},
    {".or.", T_OR},
};

bool Lex(const char *s, std::vector<Token> &out) {
    int i = 0, n = (int)strlen(s);
    while (i < n) {
        char c = s[i];
        if (c == ' ' || c == '\n' || c == '\t' || c == '\r' || c == '\f') { i++; continue; }
        Token t; t.pos = i;
        if (isdigit((unsigned char)c)) {
            int j = i;
            while (j < n && isdigit((unsigned char)s[j])) j++;
            if (j < n && s[j] == '.') { j++; while (j < n && isdigit((unsigned char)s[j])) j++; }
            if (j < n && (s[j] == 'e' || s[j] == 'E')) {
                int k = j + 1;
                if (k < n && (s[k] == '+' || s[k] == '-')) k++;
                if (k < n && isdigit((unsigned char)s[k])) {
                    while (k < n && isdigit((unsigned char)s[k])) k++;
                    j = k;
                }
            }
            t.kind = T_NUM; t.text.assign(s + i, j - i);
            t.value = atof(t.text.c_str());
            out.push_back(t); i = j; continue;
        }
        if (isalpha((unsigned char)c) || c == '_') {
            int j = i;
            while (j < n && (isalnum((unsigned char)s[j]) || s[j] == '_')) j++;
            t.text.assign(s + i, j - i);
            t.kind = T_SYM;
            for (const Keyword &kw : kWords)
                if (t.text == kw.word) { t.kind = kw.kind; t.func = kw.func; break; }
            out.push_back(t); i = j; continue;
        }
        if (c == '.') {
            bool hit = false;
            for (auto &d : kDotted) {
                size_t L = strlen(d.text);
                if (strncmp(s + i, d.text, L) == 0) { t.kind = d.kind; i += (int)L; hit = true; break; }
            }
            if (!hit) { t.kind = T_BAD; t.text = "."; out.push_back(t); return false; }
            out.push_back(t); continue;
        }
        auto two = [&](const char *p) { return i + 1 < n && s[i] == p[0] && s[i + 1] == p[1]; };
        if (two("<=")) { t.kind = T_LEQ; i += 2; }
        else if (two(">=")) { t.kind = T_GEQ; i += 2; }
        else if (two("==")) { t.kind = T_EQ; i += 2; }
        else if (two("!=")) { t.kind = T_NEQ; i += 2; }
        else if (two("&&")) { t.kind = T_AND; i += 2; }
        else if (two("||")) { t.kind = T_OR; i += 2; }
        else {
            switch (c) {
                case '<': t.kind = T_LT; break;
                case '>': t.kind = T_GT; break;
                case '~': t.kind = T_NOT; break;
                case '+': t.kind = T_PLUS; break;
                case '-': t.kind = T_MINUS; break;
                case '*': t.kind = T_TIMES; break;
                case '/': t.kind = T_DIV; break;
                case '^': t.kind = T_POW; break;
                case '(': t.kind = T_LP; break;
                case ')': t.kind = T_RP; break;
                default:
                    t.kind = T_BAD; t.text.assign(1, c);
                    printf("bad \"%c\"\n", c);
                    out.push_back(t);
                    return false;
            }
            i++;
        }
        out.push_back(t);
    }
    Token e; e.kind = T_END; e.pos = n; out.push_back(e);
    return true;
}

class Parser {
  public:
    Parser(const std::vector<Token> &toks, TermTable &tab) : t_(toks), tab_(tab) {}

    bool ParseAll() {
        // anyexpr : numexpr END | binexpr END   (LEMS_Expr.y:102-105)
        Mark m = Save();
        int root = -1;
        if (Boolean(root) && Peek() == T_END) { tab_.expression_root = root; return true; }
        Restore(m);
        if (Numeric(root) && Peek() == T_END) { tab_.expression_root = root; return true; }
        return false;
    }
    int FailPos() const { return far_ < (int)t_.size() ? t_[far_].pos : 0; }

  private:
    struct Mark { size_t p, nterms, nsyms; };
    const std::vector<Token> &t_;
    TermTable &tab_;
    size_t p_ = 0;
    int far_ = 0;

    Mark Save() const { return {p_, tab_.terms.size(), tab_.symbol_refs.size()}; }
    void Restore(const Mark &m) {
        p_ = m.p;
        tab_.terms.resize(m.nterms, Term(0.0));
        tab_.symbol_refs.resize(m.nsyms);
    }
    Tok Peek() const { return t_[p_].kind; }
    void Next() { p_++; if ((int)p_ > far_) far_ = (int)p_; }
    bool Accept(Tok k) { if (Peek() == k) { Next(); return true; } return false; }

    // ---- boolean expressions: or < and < not < comparison ----
    bool Boolean(int &out) {
        int l;
        if (!BoolAnd(l)) return false;
        while (Peek() == T_OR) {
            Next();
            int r;
            if (!BoolAnd(r)) return false;
            l = tab_.add(Term(Term::OR, l, r));
        }
        out = l; return true;
    }
    bool BoolAnd(int &out) {
        int l;
        if (!BoolUnary(l)) return false;
        while (Peek() == T_AND) {
            Next();
            int r;
            if (!BoolUnary(r)) return false;
            l = tab_.add(Term(Term::AND, l, r));
        }
        out = l; return true;
    }
    bool BoolUnary(int &out) {
        if (Peek() == T_NOT) {
            Next();
            int r;
            if (!BoolUnary(r)) return false;
            out = tab_.add(Term(Term::NOT, r));
            return true;
        }
        // numexpr RELOP numexpr, else '(' binexpr ')'
        Mark m = Save();
        int l;
        if (Numeric(l)) {
            Term::Type op = Term::NONE;
            switch (Peek()) {
                case T_LEQ: op = Term::LEQ; break;
                case T_GEQ: op = Term::GEQ; break;
                case T_LT: op = Term::LT; break;
                case T_GT: op = Term::GT; break;
                case T_EQ: op = Term::EQ; break;
                case T_NEQ: op = Term::NEQ; break;
                default: break;
            }
            if (op != Term::NONE) {
                Next();
                int r;
                if (Numeric(r)) { out = tab_.add(Term(op, l, r)); return true; }
            }
        }
        Restore(m);
        if (Peek() == T_LP) {
            Next();
            int inner;
            if (Boolean(inner) && Accept(T_RP)) { out = inner; return true; }
        }
        Restore(m);
        return false;
    }

    // ---- numeric expressions: + - < * / < ^ (right) < unary +- ----
    bool Numeric(int &out) {
        int l;
        if (!Product(l)) return false;
        while (Peek() == T_PLUS || Peek() == T_MINUS) {
            Term::Type op = Peek() == T_PLUS ? Term::PLUS : Term::MINUS;
            Next();
            int r;
            if (!Product(r)) return false;
            l = tab_.add(Term(op, l, r));
        }
        out = l; return true;
    }
    bool Product(int &out) {
        int l;
        if (!Power(l)) return false;
        while (Peek() == T_TIMES || Peek() == T_DIV) {
            Term::Type op = Peek() == T_TIMES ? Term::TIMES : Term::DIVIDE;
            Next();
            int r;
            if (!Power(r)) return false;
            l = tab_.add(Term(op, l, r));
        }
        out = l; return true;
    }
    bool Power(int &out) {
        int base;
        if (!Unary(base)) return false;
        if (Peek() == T_POW) {
            Next();
            int expo;
            if (!Power(expo)) return false;
            out = tab_.add(Term(Term::POWER, base, expo));
            return true;
        }
        out = base; return true;
    }
    bool Unary(int &out) {
        if (Peek() == T_MINUS || Peek() == T_PLUS) {
            Term::Type op = Peek() == T_MINUS ? Term::UMINUS : Term::UPLUS;
            Next();
            int r;
            if (!Unary(r)) return false;
            out = tab_.add(Term(op, r));
            return true;
        }
        return Primary(out);
    }
    bool Primary(int &out) {
        const Token &tk = t_[p_];
        switch (tk.kind) {
            case T_NUM: Next(); out = tab_.add(Term(tk.value)); return true;
            case T_SYM: Next(); out = tab_.addSymbol(tk.text.c_str()); return true;
            case T_LP: {
                Next();
                int inner;
                if (!Numeric(inner) || !Accept(T_RP)) return false;
                out = inner; return true;
            }
            case T_FUNC: {
                Term::Type f = tk.func;
                Next();
                if (!Accept(T_LP)) return false;
                Mark m = Save();
                int arg;
                if (Numeric(arg) && Accept(T_RP)) { out = tab_.add(Term(f, arg)); return true; }
                if (f != Term::INT) return false;
                // int( binexpr )   (LEMS_Expr.y:154)
                Restore(m);
                if (Boolean(arg) && Accept(T_RP)) { out = tab_.add(Term(f, arg)); return true; }
                return false;
            }
            default: return false;
        }
    }
};

const char *TypeName(Term::Type t) {
    switch (t) {
        case Term::PLUS: return "+"; case Term::MINUS: return "-";
        case Term::TIMES: return "*"; case Term::DIVIDE: return "/";
        case Term::POWER: return "^"; case Term::LEQ: return "<=";
        case Term::GEQ: return ">="; case Term::LT: return "<";
        case Term::GT: return ">"; case Term::EQ: return "==";
        case Term::NEQ: return "!="; case Term::AND: return "and";
        case Term::OR: return "or"; case Term::UMINUS: return "-";
        case Term::UPLUS: return "+"; case Term::NOT: return "not";
        case Term::ABS: return "abs"; case Term::SQRT: return "sqrt";
        case Term::SIN: return "sin"; case Term::COS: return "cos";
        case Term::TAN: return "tan"; case Term::SINH: return "sinh";
        case Term::COSH: return "cosh"; case Term::TANH: return "tanh";
        case Term::EXP: return "exp"; case Term::LOG10: return "log10";
        case Term::LN: return "ln"; case Term::CEIL: return "ceil";
        case Term::FLOOR: return "floor"; case Term::RANDOM: return "random";
        case Term::HFUNC: return "H"; case Term::INT: return "int";
        default: return "?";
    }
}

}  // namespace

bool ParseLemsExpression(const char *sInput, TermTable &tab) {
    std::vector<Token> toks;
    if (!Lex(sInput, toks)) {
        printf("Error: invalid character in expression\n%s\n", sInput);
        return false;
    }
    Parser p(toks, tab);
    if (!p.ParseAll()) {
        int at = p.FailPos();
        printf("Error on byte %d: syntax error\n%s\n", at + 1, sInput);
        for (int i = 0; i < at; i++) printf(" ");
        printf("^\n");
        return false;
    }
    return true;
}

void TermTable::printTree(const TermTable &tab, int node, int tabDepth) {
    const Term &term = tab[node];
    for (int i = 0; i < tabDepth; i++) printf("    ");
    printf("< %d >\n", node);
    for (int i = 0; i < tabDepth; i++) printf("    ");
    if (term.type == Term::VALUE) { printf("%f\n", term.value); return; }
    if (term.type == Term::SYMBOL) {
        printf("#%d %s\n", term.symbol, tab.symbol_refs[term.symbol].c_str());
        return;
    }
    printf("%s \n", TypeName(term.type));
    if (term.isBinaryOperator()) printTree(tab, term.left, tabDepth + 1);
    if (term.isBinaryOperator() || term.isUnary()) printTree(tab, term.right, tabDepth + 1);
}
