/* Empty stand-in: the hot-path sources use no Hypre declarations. */
