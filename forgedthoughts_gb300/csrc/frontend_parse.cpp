// `.ft` lexer and recursive-descent parser.
//
// Token set and grammar follow crates/forgedthoughts/src/lexer.rs:1-199 and
// crates/forgedthoughts/src/parser.rs:25-800: numbers are digit/dot runs
// parsed as f64 (no exponent form), `#rgb`/`#rrggbb` colours become vec3
// object literals with channels /255 (parser.rs:760-800), `//` comments, and
// expression precedence add/sub/intersect < mul/div < unary minus < postfix
// (member, call).
#include <cctype>
#include <cstdlib>
#include <sstream>

#include "frontend.h"

namespace ftfe {
namespace {

enum class Tok {
  Let, Var, Fn, Return, Import, Export, Ident, String, HexColor, Number,
  Equal, Semicolon, Colon, Comma, Dot, Plus, Minus, Amp, Star, Slash,
  LParen, RParen, LBracket, RBracket, LBrace, RBrace
};

struct Token {
  Tok kind;
  std::string text;
  double number = 0.0;
  size_t start = 0;
};

[[noreturn]] void parse_fail(const std::string& msg) { throw FrontendError(FT_ERR_PARSE, msg); }

bool is_ident_start(char c) { return std::isalpha(static_cast<unsigned char>(c)) || c == '_'; }
bool is_ident_continue(char c) { return std::isalnum(static_cast<unsigned char>(c)) || c == '_'; }

std::vector<Token> tokenize(const std::string& in) {
  std::vector<Token> out;
  size_t i = 0, n = in.size();
  auto simple = [&](Tok k, size_t at) { out.push_back(Token{k, "", 0.0, at}); };
  while (i < n) {
    char c = in[i];
    size_t at = i;
    if (c == ' ' || c == '\t' || c == '\r' || c == '\n') { ++i; continue; }
    if (c == '"') {
      std::string value;
      bool closed = false;
      ++i;
      while (i < n) {
        char d = in[i++];
        if (d == '"') { closed = true; break; }
        if (d == '\\') {
          if (i >= n) break;
          char e = in[i++];
          switch (e) {
            case 'n': value.push_back('\n'); break;
            case 'r': value.push_back('\r'); break;
            case 't': value.push_back('\t'); break;
            default: value.push_back(e); break;
          }
          continue;
        }
        value.push_back(d);
      }
      if (!closed) parse_fail("unexpected character '\"' at byte " + std::to_string(at));
      out.push_back(Token{Tok::String, value, 0.0, at});
      continue;
    }
    if (c == '#') {
      std::string digits;
      ++i;
      while (i < n && std::isxdigit(static_cast<unsigned char>(in[i]))) {
        digits.push_back(static_cast<char>(std::tolower(static_cast<unsigned char>(in[i]))));
        ++i;
      }
      if (!(digits.size() == 3 || digits.size() == 6))
        parse_fail("invalid hex color '#" + digits + "' at byte " + std::to_string(at));
      out.push_back(Token{Tok::HexColor, digits, 0.0, at});
      continue;
    }
    if (c == '/') {
      if (i + 1 < n && in[i + 1] == '/') {
        while (i < n && in[i] != '\n') ++i;
        continue;
      }
      simple(Tok::Slash, at); ++i; continue;
    }
    switch (c) {
      case '=': simple(Tok::Equal, at); ++i; continue;
      case ';': simple(Tok::Semicolon, at); ++i; continue;
      case ':': simple(Tok::Colon, at); ++i; continue;
      case ',': simple(Tok::Comma, at); ++i; continue;
      case '.': simple(Tok::Dot, at); ++i; continue;
      case '+': simple(Tok::Plus, at); ++i; continue;
      case '-': simple(Tok::Minus, at); ++i; continue;
      case '&': simple(Tok::Amp, at); ++i; continue;
      case '*': simple(Tok::Star, at); ++i; continue;
      case '(': simple(Tok::LParen, at); ++i; continue;
      case ')': simple(Tok::RParen, at); ++i; continue;
      case '[': simple(Tok::LBracket, at); ++i; continue;
      case ']': simple(Tok::RBracket, at); ++i; continue;
      case '{': simple(Tok::LBrace, at); ++i; continue;
      case '}': simple(Tok::RBrace, at); ++i; continue;
      default: break;
    }
    if (is_ident_start(c)) {
      std::string lex;
      while (i < n && is_ident_continue(in[i])) lex.push_back(in[i++]);
      Tok k = Tok::Ident;
      if (lex == "let") k = Tok::Let;
      else if (lex == "var") k = Tok::Var;
      else if (lex == "fn") k = Tok::Fn;
      else if (lex == "return") k = Tok::Return;
      else if (lex == "import") k = Tok::Import;
      else if (lex == "export") k = Tok::Export;
      out.push_back(Token{k, k == Tok::Ident ? lex : std::string(), 0.0, at});
      continue;
    }
    if (std::isdigit(static_cast<unsigned char>(c))) {
      std::string lex;
      while (i < n && (std::isdigit(static_cast<unsigned char>(in[i])) || in[i] == '.')) lex.push_back(in[i++]);
      // Rust's f64 parser rejects a second '.'; strtod would stop early.
      size_t dots = 0;
      for (char d : lex) dots += d == '.';
      char* end = nullptr;
      double v = std::strtod(lex.c_str(), &end);
      if (dots > 1 || end != lex.c_str() + lex.size())
        parse_fail("invalid number '" + lex + "' at byte " + std::to_string(at));
      out.push_back(Token{Tok::Number, "", v, at});
      continue;
    }
    parse_fail(std::string("unexpected character '") + c + "' at byte " + std::to_string(at));
  }
  return out;
}

ExprP make_expr(Expr e) { return std::make_shared<const Expr>(std::move(e)); }

class Parser {
 public:
  explicit Parser(std::vector<Token> t) : toks_(std::move(t)) {}

  std::vector<Stmt> program() {
    std::vector<Stmt> out;
    while (pos_ < toks_.size()) out.push_back(statement());
    return out;
  }

 private:
  std::vector<Token> toks_;
  size_t pos_ = 0;

  const Token* peek() const { return pos_ < toks_.size() ? &toks_[pos_] : nullptr; }
  bool match(Tok k) {
    if (pos_ < toks_.size() && toks_[pos_].kind == k) { ++pos_; return true; }
    return false;
  }
  bool match_ident(const char* s) {
    if (pos_ < toks_.size() && toks_[pos_].kind == Tok::Ident && toks_[pos_].text == s) { ++pos_; return true; }
    return false;
  }
  size_t offset() const {
    if (pos_ < toks_.size()) return toks_[pos_].start;
    return toks_.empty() ? 0 : toks_.back().start;
  }
  void expect(Tok k, const char* what) {
    if (!match(k)) parse_fail(std::string("expected ") + what + " at byte " + std::to_string(offset()));
  }
  std::string expect_ident() {
    const Token* t = peek();
    if (!t) parse_fail("unexpected end of input");
    if (t->kind != Tok::Ident) parse_fail("expected identifier at byte " + std::to_string(offset()));
    ++pos_;
    return t->text;
  }
  std::string expect_string() {
    const Token* t = peek();
    if (!t) parse_fail("unexpected end of input");
    if (t->kind != Tok::String) parse_fail("expected string literal at byte " + std::to_string(offset()));
    ++pos_;
    return t->text;
  }

  Stmt statement() {
    Stmt s;
    if (match(Tok::Import)) {
      s.kind = Stmt::Import;
      s.name = expect_string();
      if (match_ident("as")) s.alias = expect_ident();
      expect(Tok::Semicolon, ";");
      return s;
    }
    if (match(Tok::Export)) {
      s.kind = Stmt::Export;
      expect(Tok::LBrace, "{");
      if (!match(Tok::RBrace)) {
        for (;;) {
          s.path.push_back(expect_ident());
          if (match(Tok::Comma)) continue;
          expect(Tok::RBrace, "}");
          break;
        }
      }
      expect(Tok::Semicolon, ";");
      return s;
    }
    if (match_ident("material")) return block_def(Stmt::Material);
    if (match_ident("sdf")) return block_def(Stmt::Sdf);
    if (match_ident("skeleton")) return skeleton_def();
    if (match_ident("environment")) return block_def(Stmt::Environment);
    if (match(Tok::Fn)) {
      s.kind = Stmt::Function;
      s.fn = std::make_shared<FunctionDef>();
      s.fn->name = expect_ident();
      s.fn->params = params();
      s.fn->body = fn_body_or_expr();
      s.name = s.fn->name;
      return s;
    }
    if (match(Tok::Let)) return binding(false);
    if (match(Tok::Var)) return binding(true);
    // assignment: ident(.ident)* = expr ;
    s.kind = Stmt::Assign;
    s.path.push_back(expect_ident());
    while (match(Tok::Dot)) s.path.push_back(expect_ident());
    expect(Tok::Equal, "=");
    s.expr = expr();
    expect(Tok::Semicolon, ";");
    return s;
  }

  Stmt binding(bool mut) {
    Stmt s;
    s.kind = Stmt::Binding;
    s.mutable_ = mut;
    s.name = expect_ident();
    expect(Tok::Equal, "=");
    s.expr = expr();
    expect(Tok::Semicolon, ";");
    return s;
  }

  std::vector<FnStmt> fn_body_or_expr() {
    if (match(Tok::Equal)) {
      FnStmt r;
      r.is_return = true;
      r.expr = expr();
      expect(Tok::Semicolon, ";");
      return {r};
    }
    return fn_body();
  }

  std::vector<FnStmt> fn_body() {
    expect(Tok::LBrace, "{");
    std::vector<FnStmt> body;
    while (!match(Tok::RBrace)) {
      FnStmt st;
      if (match(Tok::Let)) {
        st.name = expect_ident();
        expect(Tok::Equal, "=");
        st.expr = expr();
        expect(Tok::Semicolon, ";");
        body.push_back(st);
        continue;
      }
      if (match(Tok::Return)) {
        st.is_return = true;
        st.expr = expr();
        expect(Tok::Semicolon, ";");
        body.push_back(st);
        continue;
      }
      parse_fail("expected let or return at byte " + std::to_string(offset()));
    }
    return body;
  }

  std::vector<std::string> params() {
    expect(Tok::LParen, "(");
    std::vector<std::string> ps;
    if (!match(Tok::RParen)) {
      for (;;) {
        ps.push_back(expect_ident());
        if (match(Tok::Comma)) continue;
        expect(Tok::RParen, ")");
        break;
      }
    }
    return ps;
  }

  // material / sdf / environment blocks (parser.rs:124-314)
  Stmt block_def(Stmt::Kind kind) {
    Stmt s;
    s.kind = kind;
    s.block = std::make_shared<BlockDef>();
    s.block->name = expect_ident();
    s.name = s.block->name;
    expect(Tok::LBrace, "{");
    std::string model;
    while (!match(Tok::RBrace)) {
      BlockStmt bs;
      if (match(Tok::Let)) {
        bs.kind = BlockStmt::Binding;
        bs.name = expect_ident();
        expect(Tok::Equal, "=");
        bs.expr = expr();
        expect(Tok::Semicolon, ";");
        s.block->statements.push_back(bs);
        continue;
      }
      if (match(Tok::Fn)) {
        bs.kind = BlockStmt::Function;
        bs.name = expect_ident();
        bs.params = params();
        bs.body = fn_body_or_expr();
        s.block->statements.push_back(bs);
        continue;
      }
      std::string field = expect_ident();
      if (kind == Stmt::Material && match(Tok::Equal)) {
        bs.kind = BlockStmt::Property;
        bs.name = field;
        bs.expr = expr();
        expect(Tok::Semicolon, ";");
        s.block->statements.push_back(bs);
        continue;
      }
      if (kind == Stmt::Material && field == "model") {
        expect(Tok::Colon, ":");
        model = expect_ident();
        expect(Tok::Semicolon, ";");
        continue;
      }
      if (field == "name" || field == "description" || field == "tags" || field == "params") {
        expect(Tok::Colon, ":");
        expr();
        expect(Tok::Semicolon, ";");
        continue;
      }
      parse_fail(std::string("expected ") +
                 (kind == Stmt::Material ? "let, fn, property assignment, or model" : "let, fn, or metadata field") +
                 " at byte " + std::to_string(offset()));
    }
    expect(Tok::Semicolon, ";");
    s.block->model = model.empty() ? "Standard" : model;
    return s;
  }

  // Skeleton blocks are parsed and dropped: they only drive authoring-time IK.
  Stmt skeleton_def() {
    Stmt s;
    s.kind = Stmt::Skeleton;
    s.name = expect_ident();
    expect(Tok::LBrace, "{");
    while (!match(Tok::RBrace)) {
      if (match(Tok::Let) || match_ident("joint")) {
        expect_ident();
        expect(Tok::Equal, "=");
        expr();
        expect(Tok::Semicolon, ";");
        continue;
      }
      if (match_ident("bone")) {
        expect_ident(); expect(Tok::Equal, "="); expect_ident(); expect(Tok::Comma, ","); expect_ident();
        expect(Tok::Semicolon, ";");
        continue;
      }
      if (match_ident("chain")) {
        expect_ident(); expect(Tok::Equal, "="); expect_ident(); expect(Tok::Comma, ",");
        expect_ident(); expect(Tok::Comma, ","); expect_ident();
        expect(Tok::Semicolon, ";");
        continue;
      }
      std::string field = expect_ident();
      if (field == "name" || field == "description" || field == "tags" || field == "params") {
        expect(Tok::Colon, ":"); expr(); expect(Tok::Semicolon, ";");
        continue;
      }
      parse_fail("expected let, joint, bone, chain, or metadata field at byte " + std::to_string(offset()));
    }
    expect(Tok::Semicolon, ";");
    return s;
  }

  ExprP expr() { return add_sub(); }

  ExprP add_sub() {
    ExprP e = mul_div();
    for (;;) {
      char op = 0;
      if (match(Tok::Plus)) op = '+';
      else if (match(Tok::Minus)) op = '-';
      else if (match(Tok::Amp)) op = '&';
      if (!op) break;
      Expr b;
      b.kind = Expr::Binary;
      b.op = op;
      b.lhs = e;
      b.rhs = mul_div();
      e = make_expr(std::move(b));
    }
    return e;
  }

  ExprP mul_div() {
    ExprP e = unary();
    for (;;) {
      char op = 0;
      if (match(Tok::Star)) op = '*';
      else if (match(Tok::Slash)) op = '/';
      if (!op) break;
      Expr b;
      b.kind = Expr::Binary;
      b.op = op;
      b.lhs = e;
      b.rhs = unary();
      e = make_expr(std::move(b));
    }
    return e;
  }

  ExprP unary() {
    if (match(Tok::Minus)) {
      Expr u;
      u.kind = Expr::Unary;
      u.op = '-';
      u.lhs = unary();
      return make_expr(std::move(u));
    }
    return postfix();
  }

  ExprP postfix() {
    ExprP e = primary();
    for (;;) {
      if (match(Tok::Dot)) {
        Expr m;
        m.kind = Expr::Member;
        m.lhs = e;
        m.text = expect_ident();
        e = make_expr(std::move(m));
        continue;
      }
      if (match(Tok::LParen)) {
        Expr c;
        c.kind = Expr::Call;
        c.lhs = e;
        if (!match(Tok::RParen)) {
          for (;;) {
            c.items.push_back(expr());
            if (match(Tok::Comma)) continue;
            expect(Tok::RParen, ")");
            break;
          }
        }
        e = make_expr(std::move(c));
        continue;
      }
      break;
    }
    return e;
  }

  std::vector<std::pair<std::string, ExprP>> object_fields() {
    std::vector<std::pair<std::string, ExprP>> fields;
    if (match(Tok::RBrace)) return fields;
    for (;;) {
      std::string key = expect_ident();
      expect(Tok::Colon, ":");
      fields.emplace_back(key, expr());
      if (match(Tok::Comma)) {
        if (match(Tok::RBrace)) return fields;
        continue;
      }
      expect(Tok::RBrace, "}");
      break;
    }
    return fields;
  }

  ExprP primary() {
    if (match(Tok::Fn)) {
      Expr f;
      f.kind = Expr::FunctionLiteral;
      f.params = params();
      f.body = fn_body_or_expr();
      return make_expr(std::move(f));
    }
    if (match(Tok::LParen)) {
      ExprP e = expr();
      expect(Tok::RParen, ")");
      return e;
    }
    if (match(Tok::LBrace)) {
      Expr o;
      o.kind = Expr::ObjectLiteral;
      o.text = "anonymous";
      o.fields = object_fields();
      return make_expr(std::move(o));
    }
    if (match(Tok::LBracket)) {
      Expr a;
      a.kind = Expr::Array;
      if (!match(Tok::RBracket)) {
        for (;;) {
          a.items.push_back(expr());
          if (match(Tok::Comma)) continue;
          expect(Tok::RBracket, "]");
          break;
        }
      }
      return make_expr(std::move(a));
    }
    const Token* t = peek();
    if (!t) parse_fail("unexpected end of input");
    switch (t->kind) {
      case Tok::String: {
        ++pos_;
        Expr s;
        s.kind = Expr::String;
        s.text = t->text;
        return make_expr(std::move(s));
      }
      case Tok::HexColor: {
        ++pos_;
        const std::string& h = t->text;
        double ch[3];
        if (h.size() == 3) {
          for (int k = 0; k < 3; ++k) {
            int v = std::stoi(h.substr(k, 1), nullptr, 16);
            ch[k] = double((v << 4) | v) / 255.0;
          }
        } else {
          for (int k = 0; k < 3; ++k) ch[k] = double(std::stoi(h.substr(2 * k, 2), nullptr, 16)) / 255.0;
        }
        Expr o;
        o.kind = Expr::ObjectLiteral;
        o.text = "vec3";
        const char* names[3] = {"x", "y", "z"};
        for (int k = 0; k < 3; ++k) {
          Expr num;
          num.kind = Expr::Number;
          num.number = ch[k];
          o.fields.emplace_back(names[k], make_expr(std::move(num)));
        }
        return make_expr(std::move(o));
      }
      case Tok::Number: {
        ++pos_;
        Expr num;
        num.kind = Expr::Number;
        num.number = t->number;
        return make_expr(std::move(num));
      }
      case Tok::Ident: {
        std::vector<std::string> segs{expect_ident()};
        while (match(Tok::Dot)) segs.push_back(expect_ident());
        if (match(Tok::LBrace)) {
          Expr o;
          o.kind = Expr::ObjectLiteral;
          std::string joined;
          for (size_t k = 0; k < segs.size(); ++k) joined += (k ? "." : "") + segs[k];
          o.text = joined;
          o.fields = object_fields();
          return make_expr(std::move(o));
        }
        Expr id;
        id.kind = Expr::Ident;
        id.text = segs[0];
        ExprP e = make_expr(std::move(id));
        for (size_t k = 1; k < segs.size(); ++k) {
          Expr m;
          m.kind = Expr::Member;
          m.lhs = e;
          m.text = segs[k];
          e = make_expr(std::move(m));
        }
        return e;
      }
      default:
        parse_fail("unexpected token at byte " + std::to_string(offset()));
    }
  }
};

}  // namespace

std::vector<Stmt> parse_program(const std::string& source) {
  Parser p(tokenize(source));
  return p.program();
}

}  // namespace ftfe
