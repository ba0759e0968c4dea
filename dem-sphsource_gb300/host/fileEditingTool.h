// Output-directory helpers of the host API (core/fileEditingTool.h:53-140 in
// the reference): solverBase clears a case's old frames before writing new ones.
#pragma once
#include <filesystem>
#include <string>
#include <system_error>

namespace demsph {
// Deletes the regular files directly in `dir` whose extension is `ext`;
// returns how many were removed (0 when the directory does not exist).
inline int removeFilesWithExtension(const std::string& dir, const char* ext)
{
    namespace fs = std::filesystem;
    std::error_code ec;
    int removed = 0;
    for (fs::directory_iterator it(dir, ec), end; !ec && it != end; it.increment(ec)) {
        if (it->is_regular_file(ec) && it->path().extension() == ext && fs::remove(it->path(), ec)) ++removed;
    }
    return removed;
}
}  // namespace demsph

inline int removeVtuFiles(const std::string& dir) { return demsph::removeFilesWithExtension(dir, ".vtu"); }
inline int removeDatFiles(const std::string& dir) { return demsph::removeFilesWithExtension(dir, ".dat"); }
