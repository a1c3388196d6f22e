// Stand-in for Boost.ConceptCheck: compile-time concept assertions become no-ops.
#pragma once
#define BOOST_CONCEPT_ASSERT(x)
