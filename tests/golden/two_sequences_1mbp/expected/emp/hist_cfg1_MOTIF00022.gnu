set output "hist_cfg1_MOTIF00022.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-90.9062:21.9997]
set yrange [0:2548]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_cfg1_MOTIF00022.dat" using 1:2 title 'MOTIF00022 (cfg1)' with boxes
