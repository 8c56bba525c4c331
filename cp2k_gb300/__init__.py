"""GB300-native CP2K grid collocate/integrate backend (host package)."""
