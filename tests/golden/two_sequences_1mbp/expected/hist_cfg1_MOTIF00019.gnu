set output "hist_cfg1_MOTIF00019.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-92.4762:26.0019]
set yrange [0:178019]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_cfg1_MOTIF00019.dat" using 1:2 title 'MOTIF00019 (cfg1)' with boxes
