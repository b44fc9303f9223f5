// Stand-in: boost::any as std::any.
#pragma once
#include <any>
namespace boost { using std::any; using std::any_cast; }
