// Project-written stand-in: the reference only names boost::shared_ptr in
// typedefs of out-of-scope index types.  Test infrastructure only.
#pragma once
#include <memory>
namespace boost { using std::shared_ptr; }
