/* Forward declaration only: the hot-path sources never use JSON values. */
#ifndef REFSHIM_JSON_H
#define REFSHIM_JSON_H
namespace Json { class Value; }
#endif
