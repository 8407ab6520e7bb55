"""GB300-native iterative stockholder partitioning (MBIS, GISA, aLISA, gLISA)."""
