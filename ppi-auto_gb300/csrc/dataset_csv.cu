// dataset_csv.cu -- PPI's training CSV read straight into the evaluator's
// column-major device layout (host code).
//
// PPI reads its dataset with read() of src/main.cc:32-122 into float** rows
// and hands those to acc_interpret_init; this reader follows the same rules so
// that the same file gives the same records, and writes the columns the
// device layout wants directly (no row array, no transpose of row pointers):
//   * a line that is empty or starts with '#' is skipped (it still counts in
//     the line numbers of messages);
//   * tokens are separated by ',' (std::getline: a trailing ',' adds no
//     token, ",," gives an empty token);
//   * the first counted line fixes the column count; it is a header when its
//     LAST token is not a number (counting pass, :46-58), and in the reading
//     pass a line is a header when its FIRST token is not a number (:74-80);
//   * a token is a number as util::StringTo<float> (src/util/Util.h:46-49)
//     reads it: `std::istringstream >> float`, see parse_float below;
//   * a value that does not parse, or is NaN or infinite: "Invalid input at
//     line L, column C." (status 2); a data line with another column count:
//     "Line 'L' has 'J' columns but the expected number is 'N'." (status 1).
// Where the reference is undefined the reader reports an error instead: a
// data line with more columns than the first line (the reference writes past
// its row before it checks), and a file whose two passes disagree on which
// line is the header (the reference then writes past its row array or leaves
// its last row unset).
#include <cctype>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "ppi_internal.cuh"

namespace ppi {
namespace {

// `std::istringstream(s) >> f` in the "C" locale, as libstdc++ implements it
// (num_get::_M_extract_float, then strtof): white space is skipped; the
// longest prefix of the form [sign] digits [. digits] [e [sign] digits] is
// collected (an exponent only after a mantissa digit, one decimal point
// before it); the read fails unless strtof consumes all of that prefix, and
// fails on an overflow to infinity.  Whatever follows the prefix is ignored,
// so "1.5abc" reads 1.5 while "1e" and "." fail.
bool parse_float(const std::string& s, float* out) {
   size_t i = 0;
   while (i < s.size() && std::isspace((unsigned char)s[i])) ++i;
   std::string x;
   if (i < s.size() && (s[i] == '+' || s[i] == '-')) x += s[i++];
   bool mantissa = false, dec = false, sci = false;
   while (i < s.size()) {
      const char c = s[i];
      if (c >= '0' && c <= '9') {
         x += c;
         mantissa = true;
      } else if (c == '.' && !dec && !sci) {
         x += '.';
         dec = true;
      } else if ((c == 'e' || c == 'E') && !sci && mantissa) {
         x += 'e';
         sci = true;
         if (i + 1 < s.size() && (s[i + 1] == '+' || s[i + 1] == '-')) x += s[++i];
      } else {
         break;
      }
      ++i;
   }
   if (x.empty()) return false;
   char* end = nullptr;
   errno = 0;
   const float v = std::strtof(x.c_str(), &end);
   if (end == x.c_str() || *end != '\0') return false;
   if (std::isinf(v)) return false;
   *out = v;
   return true;
}

std::vector<std::string> split_commas(const std::string& line) {
   std::vector<std::string> t;
   size_t b = 0;
   while (b < line.size()) {
      const size_t e = line.find(',', b);
      if (e == std::string::npos) {
         t.push_back(line.substr(b));
         break;
      }
      t.push_back(line.substr(b, e - b));
      b = e + 1;
   }
   return t;
}

}  // namespace

// Reads `path`; on success fills rows x cols and, when colmajor is given,
// the values at colmajor[c * ld + r] (ld >= rows).  Returns 0, 1 (column
// count) or 2 (open / value), with the reference's message in *msg.
int read_csv(const char* path, std::vector<float>* colmajor, int pad, int* rows, int* cols,
             std::string* msg) {
   FILE* f = std::fopen(path, "rb");
   if (!f) {
      *msg = std::string("Failed to open dataset file '") + path +
             "' (use '-d dataset', where dataset is the path of the training CSV file)";
      return 2;
   }
   std::string text;
   char buf[1 << 16];
   for (size_t n; (n = std::fread(buf, 1, sizeof buf, f)) > 0;) text.append(buf, n);
   std::fclose(f);
   std::vector<std::string> lines;
   for (size_t b = 0; b <= text.size();) {
      size_t e = text.find('\n', b);
      if (e == std::string::npos) {
         if (b < text.size()) lines.push_back(text.substr(b));
         break;
      }
      lines.push_back(text.substr(b, e - b));
      b = e + 1;
   }
   auto counted = [](const std::string& l) { return !l.empty() && l[0] != '#'; };
   // counting pass: the first counted line gives the columns and, by its
   // last token, whether it is a header
   int ncol = 0, nlin = 0;
   bool header = true;
   for (const std::string& l : lines) {
      if (!counted(l)) continue;
      if (header) {
         const std::vector<std::string> t = split_commas(l);
         ncol = (int)t.size();
         float tmp;
         // the reference tests the string its last std::getline left: the
         // last token, or the empty string when the line ends with ',' (that
         // call starts by erasing it, then finds nothing)
         const bool trailing = !l.empty() && l.back() == ',';
         if (parse_float(trailing || t.empty() ? std::string() : t.back(), &tmp)) header = false;
      }
      if (header) header = false;
      else ++nlin;
   }
   const int ld = pad > 1 ? (nlin + pad - 1) / pad * pad : nlin;
   if (colmajor) colmajor->assign((size_t)ld * (size_t)ncol, 0.0f);
   // reading pass
   header = true;
   int i = 0;
   for (size_t k = 0; k < lines.size(); ++k) {
      const std::string& l = lines[k];
      if (!counted(l)) continue;
      const std::vector<std::string> t = split_commas(l);
      int j = 0;
      for (const std::string& tok : t) {
         float v;
         if (header) {
            if (!parse_float(tok, &v)) break;   // a header line
            header = false;
         }
         if (!parse_float(tok, &v) || std::isnan(v) || std::isinf(v)) {
            *msg = "Invalid input at line " + std::to_string(k + 1) + ", column " + std::to_string(j + 1) + ".";
            return 2;
         }
         if (j >= ncol || i >= nlin) {
            *msg = j >= ncol ? "Line '" + std::to_string(k + 1) + "' has more columns than the expected number '" +
                                   std::to_string(ncol) + "'."
                             : std::string("the header line is not the same in both passes of the reader");
            return j >= ncol ? 1 : 2;
         }
         if (colmajor) (*colmajor)[(size_t)j * ld + i] = v;
         ++j;
      }
      if (!header && ncol != j) {
         *msg = "Line '" + std::to_string(k + 1) + "' has '" + std::to_string(j) +
                "' columns but the expected number is '" + std::to_string(ncol) + "'.";
         return 1;
      }
      if (header) header = false;
      else ++i;
   }
   if (i != nlin) {
      *msg = "the header line is not the same in both passes of the reader";
      return 2;
   }
   *rows = nlin;
   *cols = ncol;
   return 0;
}

}  // namespace ppi

extern "C" ppi_status ppi_csv_read(const char* path, float* colmajor, int64_t capacity, int32_t ld,
                                   int32_t* nlin, int32_t* ncol, char* message, int32_t message_len) {
   if (!path || !nlin || !ncol) return PPI_ERR_INVALID_ARGUMENT;
   std::vector<float> cm;
   std::string msg;
   int rows = 0, cols = 0;
   const int rc = ppi::read_csv(path, &cm, 1, &rows, &cols, &msg);
   if (message && message_len > 0) {
      std::strncpy(message, msg.c_str(), (size_t)message_len - 1);
      message[message_len - 1] = '\0';
   }
   if (rc != 0) return PPI_ERR_INVALID_ARGUMENT;
   *nlin = rows;
   *ncol = cols;
   if (!colmajor) return PPI_OK;
   if (ld < rows || (int64_t)ld * cols > capacity) return PPI_ERR_INVALID_ARGUMENT;
   for (int c = 0; c < cols; ++c)
      for (int r = 0; r < rows; ++r) colmajor[(size_t)c * ld + r] = cm[(size_t)c * rows + r];
   return PPI_OK;
}
