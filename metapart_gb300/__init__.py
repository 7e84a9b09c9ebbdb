"""GB300-native MetaPart read-partitioning path (genFastqIdx -> genHistograms -> metapart)."""
