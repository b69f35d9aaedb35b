// Assertion macros of the sharer's headers, as the solvers use them through
// gpuShareLib/Utils.h (the reference's gpuShareLib/Assert.h): the macro names
// and their meaning are part of the source interface the solvers compile
// against. With NDEBUG the checks compile to nothing, except ASSERT_OR_DO,
// which still evaluates its expression.
#ifndef GPUSHARESAT_GB300_ASSERT_H
#define GPUSHARESAT_GB300_ASSERT_H

#include <assert.h>
#include <stdio.h>
#include <stdlib.h>

#include <iostream>

// Prints "name: value " to stdout.
#define PRINTN(x_) \
    { std::cout << #x_ ": " << (x_) << " "; }

#ifdef NDEBUG
#define THROW() exit(1)
#else
#define THROW() assert(false)
#endif

// Prints the location and what msg_ prints, then stops.
#define THROW_ERROR(msg_)                                     \
    {                                                         \
        printf("Error in %s:%d: ", __FILE__, __LINE__);       \
        msg_;                                                 \
        printf("\n");                                         \
        THROW();                                              \
    }

#ifndef NDEBUG

#define ASSERT_OR_DO(e_) assert(e_);
#define ASSERT(e_) \
    if (!(e_)) THROW_ERROR(printf("assertion failed: " #e_ "\n"));
#define ASSERT_MSG(e_, msg_) \
    if (!(e_)) THROW_ERROR(printf("assertion failed: " #e_ " message: "); msg_);
#define PRINT_VALUES_MSG(a_, b_, msg_)                           \
    std::cout << " values are " << (a_) << " and " << (b_) << " "; \
    msg_;                                                        \
    std::cout << std::endl;
#define ASSERT_OP_MSG(a_, op_, b_, msg_) ASSERT_MSG((a_) op_(b_), PRINT_VALUES_MSG(a_, b_, msg_));
#define ASSERT_OP(a_, op_, b_) ASSERT_OP_MSG(a_, op_, b_, );
// min inclusive, max exclusive
#define ASSERT_BETWEEN(v_, lo_, hi_) \
    ASSERT_OP(v_, >=, lo_);          \
    ASSERT_OP(v_, <, hi_);

#else

#define ASSERT_OR_DO(e_) e_;
#define ASSERT(e_)
#define ASSERT_MSG(e_, msg_)
#define ASSERT_OP(a_, op_, b_)
#define ASSERT_OP_MSG(a_, op_, b_, msg_)
#define ASSERT_BETWEEN(v_, lo_, hi_)

#endif

#endif
